"""The entropy filter (pyfr/solvers/baseadvec/entfilter.py,
pyfr/solvers/euler/kernels/{entropylocal,entropyfilter}.mako,
pyfr/solvers/baseadvec/kernels/intcent.mako) against the oracle: three
RK45 steps of a steep density front, where the filter acts, within 1e-10
relative of the oracle's filtered steps (FP64), with and without walls."""
import numpy as np
import pytest

from oracle.fr_oracle import Discretisation, EntropyFilterOracle, rk45_step_ef

pytestmark = pytest.mark.gpu

TOL = 1e-10


@pytest.fixture(scope='module')
def built():
    import __graft_entry__ as ge
    ge.build_library()


def _relerr(a, b):
    return np.abs(a - b).max()/max(np.abs(b).max(), 1e-300)


def _cfg(bcs=False):
    from pyfr_gb300.inifile import Inifile
    cfg = Inifile()
    cfg.set('constants', 'gamma', 1.4)
    cfg.set('solver', 'order', 3)
    cfg.set('solver', 'shock-capturing', 'entropy-filter')
    cfg.set('solver-interfaces', 'riemann-solver', 'rusanov')
    cfg.set('solver-time-integrator', 'dt', 2e-3)
    cfg.set('soln-ics', 'rho', '1 + 0.8*tanh(30*(x*x + y*y - 0.25))')
    cfg.set('soln-ics', 'u', '0.5')
    cfg.set('soln-ics', 'v', '0.2')
    cfg.set('soln-ics', 'p', '1 + 0.5*tanh(30*(x*x + y*y - 0.25))')
    if bcs:
        for name in ('ylo', 'yhi'):
            cfg.set(f'soln-bcs-{name}', 'type', 'slp-adia-wall')
    return cfg


def _oracle(mesh, e):
    from pyfr_gb300.shapes import get_shape
    from tests.oracle_util import basis_of, ops_from_shape
    s = get_shape('quad', 3)
    lhs, rhs = mesh.con
    bcs = [(np.stack([side.eidxs, side.fidxs], 1), {'type': 'slp-adia-wall'})
           for name, side in sorted(mesh.bcon.items())]
    d = Discretisation(ops_from_shape(s), basis_of(s), mesh.spts['quad'],
                       np.stack([lhs.eidxs, lhs.fidxs], 1),
                       np.stack([rhs.eidxs, rhs.fidxs], 1),
                       periods=mesh.periods, bcs=bcs)
    ub = s.ubasis
    invvdm = np.linalg.inv(ub.vdm)
    vdm_ef = np.vstack([ub.vdm.T, ub.ortho_basis_at(s.fpts).T])
    wts = invvdm[:, 0, None]/e.rcpdjac_at_np('upts')
    wts /= wts.sum(axis=0)
    ops = dict(vdm=vdm_ef, invvdm=invvdm.T, m0=s.m0, mean_wts=wts,
               degs=np.array([max(m) for m in ub.modes]))
    opts = dict(d_min=1e-6, p_min=1e-6, e_tol=1e-6, f_tol=1e-4, niters=2,
                order=3, linearise=False)
    return d, EntropyFilterOracle(d, ops, opts, 1.4)


@pytest.mark.parametrize('walls', [False, True])
def test_entropy_filter_steps(built, walls):
    from pyfr_gb300.backend import B200Backend
    from pyfr_gb300.integrators import RKVdH2Integrator
    from pyfr_gb300.mesh import box, periodic_box
    from pyfr_gb300.solvers.elements import EulerElements
    from pyfr_gb300.solvers.system import EulerSystem
    mesh = box('quad', 8, -1.0, 1.0, (True, False)) if walls else \
        periodic_box('quad', 8, -1.0, 1.0)
    cfg = _cfg(walls)
    intg = RKVdH2Integrator(B200Backend(cfg), EulerSystem, mesh, cfg)

    # The oracle from the same initial state, with the same preproc
    e = EulerElements('quad', mesh.spts['quad'], cfg)
    d, ef = _oracle(mesh, e)
    u = e.set_ics_from_cfg()
    ef.filter(u)
    ef.local(u)
    ef.exchange()
    ef.exchange_bcs(u)

    for _ in range(3):
        u = rk45_step_ef(lambda x: d.rhs_euler(x, dict(gamma=1.4)), u, 2e-3,
                         ef)
    intg.run_steps(3)
    (got,) = intg.soln
    assert _relerr(got, u) < TOL

    # The filter acted on some elements
    fstr = intg.system._ef.ef_filter['quad'].get()[0]
    assert fstr.min() < 1.0 and fstr.max() == 1.0
    np.testing.assert_allclose(intg.system._ef.entmin['quad'].get(),
                               ef.entmin, rtol=1e-10)


def test_entropy_filter_chosen_form(built):
    """The chosen form with the entropy filter (FP32 filter on the system's
    copy of the solution, filtered elements merged back into the FP64
    solution): five steps of the steep front against the plain FP64 form.
    Without the filter the two forms agree to FP32 level (1e-5); with it
    the filter's bound checks run in FP32, so its decisions near the
    bounds may differ from FP64's and the bound is 1e-3 (relative L2);
    the filter acts."""
    from pyfr_gb300.backend import B200Backend
    from pyfr_gb300.integrators import MixedRKIntegrator, RKVdH2Integrator
    from pyfr_gb300.mesh import periodic_box
    from pyfr_gb300.solvers.system import EulerSystem
    mesh = periodic_box('quad', 8, -1.0, 1.0)

    def run(sc):
        out = []
        for single in (False, True):
            cfg = _cfg()
            cfg.set('solver', 'shock-capturing', sc)
            if single:
                cfg.set('backend', 'precision', 'single')
                cfg.set('backend-b200', 'mul-precision', 'bf16x3')
                cfg.set('backend-b200', 'split-products', '5')
                intg = MixedRKIntegrator(B200Backend(cfg), EulerSystem, mesh,
                                         cfg)
            else:
                intg = RKVdH2Integrator(B200Backend(cfg), EulerSystem, mesh,
                                        cfg)
            intg.run_steps(5)
            out.append((intg, intg.soln[0]))
        (_, b), (chosen, a) = out
        assert np.all(np.isfinite(a))
        return np.linalg.norm(a - b)/np.linalg.norm(b), chosen

    err0, _ = run('none')
    err1, chosen = run('entropy-filter')
    assert err0 < 1e-5
    assert err1 < 1e-3
    assert chosen.system._ef.ef_filter['quad'].get().min() < 1
