"""Ensembles: cases of uneven size, order and strength merged by order and
advanced in one CUDA graph per step give, case by case, the solution of
the same case advanced alone (FP64: 1e-12 relative; the only difference is
the rounding of the translated vertex coordinates) and stay within the
split-BF16 form's L2 bound of the FP64 ensemble."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def built():
    import __graft_entry__ as ge
    ge.build_library()


def _backend(prec, mul='native'):
    from pyfr_gb300.backend import B200Backend
    from pyfr_gb300.inifile import Inifile
    cfg = Inifile()
    cfg.set('backend', 'precision', prec)
    cfg.set('backend-b200', 'mul-precision', mul)
    if mul != 'native':
        cfg.set('backend-b200', 'split-products', '5')
    return B200Backend(cfg)


def test_ensemble_cases_match_standalone(built):
    from pyfr_gb300.cases import euler_vortex
    from pyfr_gb300.ensemble import Ensemble, vortex_cases
    from pyfr_gb300.integrators import RKVdH2Integrator
    from pyfr_gb300.solvers.system import EulerSystem

    cases = vortex_cases(6, seed=3, sizes=(4, 9), orders=(2, 3, 4))
    assert len({c['order'] for c in cases}) > 1
    dt = 1e-3
    ens = Ensemble(_backend('double'), cases, dt)
    ics = {}
    for g, i in zip(ens.groups, ens.intgs):
        (u0,) = i.soln
        for c, sl in zip(g.cases, g.slices):
            ics[c['case']] = u0[..., sl].copy()
    ens.run_steps(5)
    got = ens.case_solutions()

    for c in cases:
        cfg, mesh = euler_vortex(n=c['n'], order=c['order'], dt=dt)
        intg = RKVdH2Integrator(_backend('double'), EulerSystem, mesh, cfg,
                                initsoln={'quad': ics[c['case']]})
        intg.run_steps(5)
        (ref,) = intg.soln
        err = np.abs(got[c['case']] - ref).max()/np.abs(ref).max()
        assert err < 1e-12, (c, err)


def test_ensemble_chosen_form(built):
    from pyfr_gb300.ensemble import Ensemble, vortex_cases

    cases = vortex_cases(6, seed=4, sizes=(6, 12), orders=(2, 3, 4))
    dt = 1e-3
    plain = Ensemble(_backend('double'), cases, dt)
    chosen = Ensemble(_backend('single', 'bf16x3'), cases, dt, 'single',
                      mixed=True)
    plain.run_steps(10)
    chosen.run_steps(10)
    up, uc = plain.case_solutions(), chosen.case_solutions()
    for c in cases:
        a, b = uc[c['case']], up[c['case']]
        assert np.linalg.norm(a - b)/np.linalg.norm(b) <= 1e-6, c
