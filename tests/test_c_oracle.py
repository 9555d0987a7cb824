"""The C/OpenMP oracle agrees with the numpy oracle (which is pinned to
the reference's fixtures)."""
import numpy as np
import pytest

from tests.oracle_util import disc_for_mesh


@pytest.mark.parametrize('rsolver', ['rusanov', 'hllc'])
def test_c_oracle_euler(rsolver):
    from oracle.c_oracle import COracle
    from pyfr_gb300.cases import euler_vortex
    from pyfr_gb300.solvers.elements import EulerElements
    cfg, mesh = euler_vortex(n=8, order=3, rsolver=rsolver)
    u = EulerElements('quad', mesh.spts['quad'], cfg).set_ics_from_cfg()
    d = disc_for_mesh(mesh, 3)
    c = cfg.items_as('constants', float)
    ref = d.rhs_euler(u, c, rsolver)
    got = COracle(d, c, rsolver).rhs(u)
    assert np.abs(got - ref).max() <= 1e-12*np.abs(ref).max()


@pytest.mark.parametrize('beta,tau', [(0.5, 0.1), (0.0, 0.2), (-0.5, 0.0)])
def test_c_oracle_ns(beta, tau):
    from oracle.c_oracle import COracle
    from pyfr_gb300.cases import ns_tgv
    from pyfr_gb300.solvers.elements import NavierStokesElements
    cfg, mesh = ns_tgv(n=3, order=3, beta=beta, tau=tau)
    u = NavierStokesElements('hex', mesh.spts['hex'], cfg).set_ics_from_cfg()
    d = disc_for_mesh(mesh, 3, ns=True)
    c = cfg.items_as('constants', float) | cfg.items_as('solver-interfaces',
                                                       float)
    ref = d.rhs_ns(u, c)
    for variant, tol in (('strict', 1e-12), ('fast', 1e-10)):
        got = COracle(d, c, variant=variant).rhs(u)
        assert np.abs(got - ref).max() <= tol*np.abs(ref).max()
