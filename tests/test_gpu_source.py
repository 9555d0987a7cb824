"""Source terms ([solver-plugin-source], pyfr/plugins/source.py:8-31)
through this package's own systems and integrators against the oracle,
which evaluates the same expressions with numpy at the solution points.

* Plain FP64 right-hand side at t = 0.3 (negdivconf with its source
  macro), Euler and Navier-Stokes: relative max-norm 1e-10.
* The chosen form (FP32 right-hand side, split-BF16 applies, fused or
  not; with fused applies the source is added after the divergence
  apply): the RHS with the source minus the RHS without it equals the
  source at FP32 rounding.
* RK45 steps with time-dependent sources, each stage at its own time
  t + c_i dt, with and without CUDA graphs: 1e-10.
* evalsrcmacros: the bank overwritten with the source terms."""
import numpy as np
import pytest

from oracle.fr_oracle import rk45_step_t
from tests.oracle_util import (SOURCES, add_source, disc_for_mesh,
                               source_c_exprs)

pytestmark = pytest.mark.gpu

TOL = 1e-10
CONV = {2: ['rho', 'rhou', 'rhov', 'E'],
        3: ['rho', 'rhou', 'rhov', 'rhow', 'E']}


@pytest.fixture(scope='module')
def built():
    import __graft_entry__ as ge
    ge.build_library()


def _relerr(a, b):
    return np.abs(a - b).max()/max(np.abs(b).max(), 1e-300)


def _case(case, n, precision='double', src=True, **kw):
    from pyfr_gb300.cases import euler_vortex, ns_tgv
    if case == 'vortex':
        cfg, mesh = euler_vortex(n=n, order=3, precision=precision, **kw)
    else:
        cfg, mesh = ns_tgv(n=n, order=3, precision=precision, **kw)
    if src:
        add_source(cfg, case)
    return cfg, mesh


def _oracle_rhs(case, cfg, mesh):
    c = cfg.items_as('constants', float)
    if case == 'vortex':
        d = disc_for_mesh(mesh, 3)
        src = source_c_exprs(SOURCES[case], CONV[2], c)
        return lambda u, t: d.rhs_euler(u, c, t=t, src=src)
    d = disc_for_mesh(mesh, 3, ns=True)
    src = source_c_exprs(SOURCES[case], CONV[3], c)
    c = c | cfg.items_as('solver-interfaces', float)
    return lambda u, t: d.rhs_ns(u, c, t=t, src=src)


def _system(case, be, mesh, cfg):
    from pyfr_gb300.solvers.system import EulerSystem, NavierStokesSystem
    cls = EulerSystem if case == 'vortex' else NavierStokesSystem
    return cls(be, mesh, None, 2, cfg)


@pytest.mark.parametrize('case,n', [('vortex', 12), ('tgv', 3)])
def test_source_rhs_fp64(built, case, n):
    from pyfr_gb300.backend import B200Backend
    cfg, mesh = _case(case, n)
    s = _system(case, B200Backend(cfg), mesh, cfg)
    s.commit()
    assert s.has_src_macros and s.time_dependent
    s.rhs(0.3, 0, 1)
    (u,), (r,) = s.ele_scal_upts(0), s.ele_scal_upts(1)
    ref = _oracle_rhs(case, cfg, mesh)(u, 0.3)
    assert _relerr(r, ref) < TOL
    # The source is a visible part of the right-hand side
    ref0 = _oracle_rhs(case, cfg, mesh)
    assert _relerr(r, ref0(u, 0.0)) > 1e-6


@pytest.mark.parametrize('fuse', ['true', 'false'])
@pytest.mark.parametrize('case,n', [('vortex', 8), ('tgv', 4)])
def test_source_rhs_chosen_form(built, case, n, fuse):
    """The chosen form with and without the source: the difference of the
    two right-hand sides is the source at the solution points (the
    split-BF16 operator error is the same in both and cancels), to FP32
    rounding of the right-hand side (1e-5 of its scale)."""
    from oracle.fr_oracle import source_terms
    from pyfr_gb300.backend import B200Backend
    r = {}
    for src in (True, False):
        cfg, mesh = _case(case, n, precision='single', src=src)
        cfg.set('backend-b200', 'mul-precision', 'bf16x3')
        cfg.set('backend-b200', 'fuse-operators', fuse)
        s = _system(case, B200Backend(cfg), mesh, cfg)
        s.commit()
        names = {k.name for g in s.rhs_graphs(0, 1) for k in g.klist}
        assert ('srcterms' in names) == src
        s.rhs(0.3, 0, 1)
        (u,), (r[src],) = s.ele_scal_upts(0), s.ele_scal_upts(1)
        assert r[src].dtype == np.float32
    nd = 2 if case == 'vortex' else 3
    d = disc_for_mesh(mesh, 3)
    exprs = source_c_exprs(SOURCES[case], CONV[nd],
                           cfg.items_as('constants', float))
    want = source_terms(exprs, 0.3, u.astype(np.float64).transpose(1, 0, 2),
                        d.ploc_upts.transpose(1, 0, 2)).transpose(1, 0, 2)
    got = r[True].astype(np.float64) - r[False]
    assert np.abs(got - want).max() <= 1e-5*np.abs(r[False]).max()
    assert np.abs(want).max() > 1e-3


@pytest.mark.parametrize('graphs', [True, False])
@pytest.mark.parametrize('case,n', [('vortex', 12), ('tgv', 3)])
def test_rk45_time_dependent_source(built, case, n, graphs):
    from pyfr_gb300.backend import B200Backend
    from pyfr_gb300.integrators import RKVdH2Integrator
    from pyfr_gb300.solvers.system import EulerSystem, NavierStokesSystem
    cfg, mesh = _case(case, n, dt=2e-3)
    cfg.set('backend-b200', 'cuda-graphs', str(graphs).lower())
    cfg.set('solver-time-integrator', 'tstart', 0.2)
    cls = EulerSystem if case == 'vortex' else NavierStokesSystem
    intg = RKVdH2Integrator(B200Backend(cfg), cls, mesh, cfg)
    (u,) = intg.soln
    intg.run_steps(3)
    (got,) = intg.soln
    rhs = _oracle_rhs(case, cfg, mesh)
    t, dt = 0.2, intg.dt
    for _ in range(3):
        u = rk45_step_t(rhs, u, t, dt)
        t += dt
    assert _relerr(got, u) < TOL


def test_evalsrcmacros(built):
    from oracle.fr_oracle import source_terms
    from pyfr_gb300.backend import B200Backend
    cfg, mesh = _case('vortex', 12)
    s = _system('vortex', B200Backend(cfg), mesh, cfg)
    s.commit()
    s.set_time(0.7)
    (u,) = s.ele_scal_upts(0)
    s.evalsrcmacros(0)
    (got,) = s.ele_scal_upts(0)
    d = disc_for_mesh(mesh, 3)
    src = source_c_exprs(SOURCES['vortex'], CONV[2],
                         cfg.items_as('constants', float))
    want = source_terms(src, 0.7, u.transpose(1, 0, 2),
                        d.ploc_upts.transpose(1, 0, 2)).transpose(1, 0, 2)
    assert _relerr(got, want) < TOL
