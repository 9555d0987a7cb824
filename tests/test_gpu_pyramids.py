"""Pyramids on the GPU: the right-hand side on a periodic box of pyramids
(every cell cut into six about its centre), Euler and Navier-Stokes at
orders 1-4, against the oracle with the reference's pyramid operators
(1e-10 relative max-norm).  The box where hexahedra meet tetrahedra
through pyramids runs with the other mixed meshes (test_gpu_mixed.py)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-10


@pytest.fixture(scope='module')
def built():
    import __graft_entry__ as ge
    ge.build_library()


def _relerr(a, b):
    return np.abs(a - b).max()/max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize('order', [1, 2, 3, 4])
@pytest.mark.parametrize('system', ['euler', 'navier-stokes'])
def test_pyramid_box_rhs(built, golden, order, system):
    from oracle.fr_oracle import MixedDiscretisation
    from pyfr_gb300.inifile import Inifile
    from pyfr_gb300.mesh import mixed_box
    from pyfr_gb300.shapes import get_shape
    from pyfr_gb300.solvers.system import EulerSystem, NavierStokesSystem
    from tests.oracle_util import basis_of, ops_from_golden
    mesh = mixed_box(2, -1.0, 1.0, 'pyr')
    cfg = Inifile()
    gas = dict(gamma=1.4, mu=0.02, Pr=0.72, **{'ldg-beta': 0.5,
                                              'ldg-tau': 0.1})
    for k in ('gamma', 'mu', 'Pr'):
        cfg.set('constants', k, gas[k])
    cfg.set('solver', 'order', order)
    cfg.set('solver-interfaces', 'riemann-solver', 'rusanov')
    cfg.set('solver-interfaces', 'ldg-beta', 0.5)
    cfg.set('solver-interfaces', 'ldg-tau', 0.1)
    cfg.set('solver-elements-pyr', 'soln-pts', 'gauss-legendre')
    cfg.set('soln-ics', 'rho', '1 + 0.2*sin(pi*x)*cos(pi*y)*cos(pi*z)')
    cfg.set('soln-ics', 'u', '0.4 + 0.1*y')
    cfg.set('soln-ics', 'v', '-0.2 + 0.1*sin(pi*z)')
    cfg.set('soln-ics', 'w', '0.1*x')
    cfg.set('soln-ics', 'p', '1 + 0.1*cos(pi*x)')
    ns = system == 'navier-stokes'
    scls = NavierStokesSystem if ns else EulerSystem
    from pyfr_gb300.backend import B200Backend
    s = scls(B200Backend(cfg), mesh, None, 2, cfg)
    s.commit()
    s.rhs(0.0, 0, 1)
    (u,), (r,) = s.ele_scal_upts(0), s.ele_scal_upts(1)

    sh = get_shape('pyr', order, 'gauss-legendre',
                   {'quad': 'gauss-legendre', 'tri': 'alpha-opt'})
    lhs, rhs = mesh.con
    d = MixedDiscretisation(
        {'pyr': dict(ops=ops_from_golden(golden['operators'],
                                         f'pyr_p{order}_gauss-legendre', ns),
                     basis=basis_of(sh), verts=mesh.spts['pyr'])},
        zip(lhs.etypes, lhs.eidxs, lhs.fidxs),
        zip(rhs.etypes, rhs.eidxs, rhs.fidxs), periods=mesh.periods)
    ref = (d.rhs_ns if ns else d.rhs_euler)({'pyr': u}, gas)['pyr']
    assert _relerr(r, ref) < TOL
