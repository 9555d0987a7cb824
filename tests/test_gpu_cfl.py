"""The CFL controller's wave speed (pyfr/solvers/euler/kernels/wavespeed.mako,
pyfr/solvers/baseadvec/system.py:48-52,157-161) and step size
(pyfr/integrators/controllers.py:22-38) against the oracle: per-element
wave speeds within 1e-12 (FP64), the controller's dt from the maximum."""
import numpy as np
import pytest

from oracle.fr_oracle import linear_smats_djac, wavespeed

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def built():
    import __graft_entry__ as ge
    ge.build_library()


def _backend(cfg):
    from pyfr_gb300.backend import B200Backend
    return B200Backend(cfg)


def _cfl(cfg, cfl=0.4):
    cfg.set('solver-time-integrator', 'controller', 'cfl')
    cfg.set('solver-time-integrator', 'cfl', repr(cfl))
    return cfg


def _cases():
    from pyfr_gb300.cases import euler_mixed, euler_vortex, ns_tgv
    from pyfr_gb300.solvers.system import EulerSystem, NavierStokesSystem
    return {
        'vortex': (lambda: euler_vortex(n=10), EulerSystem),
        'tgv': (lambda: ns_tgv(n=4), NavierStokesSystem),
        'hex-pri': (lambda: euler_mixed(n=4, kinds='hex-pri'), EulerSystem),
        'pri-tet': (lambda: euler_mixed(n=4, kinds='pri-tet'), EulerSystem),
    }


@pytest.mark.parametrize('case', ['vortex', 'tgv', 'hex-pri', 'pri-tet'])
def test_wavespeed_matches_oracle(built, case):
    from pyfr_gb300.integrators import RKVdH2Integrator
    make, scls = _cases()[case]
    cfg, mesh = make()
    intg = RKVdH2Integrator(_backend(_cfl(cfg)), scls, mesh, cfg)
    wmax = intg.system.compute_max_wavespeed(intg.idxcurr)
    gamma = cfg.getfloat('constants', 'gamma')

    ref_max = 0
    for e, u in zip(intg.system.ele_map.values(), intg.soln):
        s, d = linear_smats_djac(e.name, mesh.spts[e.name], e.basis.upts)
        ref = wavespeed(u, s, d, gamma)
        got = e._wspd.get()[0]
        assert np.abs(got - ref).max() <= 1e-12*ref.max()
        ref_max = max(ref_max, ref.max())
    assert abs(wmax - ref_max) <= 1e-12*ref_max

    # The controller's first step: cfl/((2p + 1) max)
    t = intg.tcurr
    intg.advance_to(t + 1e-4)
    p = cfg.getint('solver', 'order')
    assert intg.dt_accepted[0] == pytest.approx(
        min(0.4/((2*p + 1)*ref_max), 1e-4), rel=1e-12)


def test_cfl_controller_tracks_the_solution(built):
    """dt is recomputed every cfl-nsteps steps from the current solution."""
    from pyfr_gb300.cases import euler_vortex
    from pyfr_gb300.integrators import RKVdH2Integrator
    from pyfr_gb300.solvers.system import EulerSystem
    cfg, mesh = euler_vortex(n=8)
    _cfl(cfg, 0.3)
    cfg.set('solver-time-integrator', 'cfl-nsteps', '2')
    intg = RKVdH2Integrator(_backend(cfg), EulerSystem, mesh, cfg)
    intg.advance_to(0.05)
    dts = intg.dt_accepted
    assert len(dts) > 4
    # (steps come in pairs of equal size, the last one clipped to t)
    for i in range(0, len(dts) - 2, 2):
        assert dts[i] == dts[i + 1]
    assert intg.tcurr == pytest.approx(0.05, abs=1e-12)
    wmax = intg.system.compute_max_wavespeed(intg.idxcurr)
    assert intg.compute_dt_cfl() == pytest.approx(0.3/(7*wmax), rel=1e-14)


def test_wavespeed_precision_forms(built):
    """The chosen form's wave speed (FP32 input on the reference-state
    transform) equals the FP64 one to FP32 precision."""
    from pyfr_gb300.cases import ns_tgv
    from pyfr_gb300.integrators import MixedRKIntegrator, RKVdH2Integrator
    from pyfr_gb300.solvers.system import NavierStokesSystem
    cfg, mesh = ns_tgv(n=4)
    plain = RKVdH2Integrator(_backend(_cfl(cfg)), NavierStokesSystem, mesh,
                             cfg)
    cfg, mesh = ns_tgv(n=4, precision='single')
    cfg.set('backend-b200', 'mul-precision', 'bf16x3')
    chosen = MixedRKIntegrator(_backend(_cfl(cfg)), NavierStokesSystem, mesh,
                               cfg)
    assert chosen.uref is not None
    a = plain.system.compute_max_wavespeed(plain.idxcurr)
    b = chosen.system.compute_max_wavespeed(chosen.idxcurr)
    assert b == pytest.approx(a, rel=1e-5)
