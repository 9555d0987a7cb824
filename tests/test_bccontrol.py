"""The surface quadrature of the boundary controllers (host side, no GPU):
on a box bounded in one direction the mass flow of a uniform momentum
through a boundary is m.n times its area, and the area-weighted mean of a
pressure linear along the boundary is its mid value (the integrals
pyfr/solvers/euler/inters.py:229-282 forms)."""
import numpy as np
import pytest

from tests.bc_cases import bc_case


def _elemap(cfg, mesh, ns):
    from pyfr_gb300.solvers.elements import EulerElements, NavierStokesElements
    cls = NavierStokesElements if ns else EulerElements
    return {et: cls(et, mesh.spts[et], cfg) for et in mesh.spts}


@pytest.mark.parametrize('kind', ['euler', 'ns'])
@pytest.mark.parametrize('qdeg', [1, 4, 7])
def test_surface_integrals(kind, qdeg):
    from pyfr_gb300.solvers.bccontrol import SurfaceIntegrator
    types = ('char-riem-inv-mass-flow', 'char-riem-inv-pressure')
    cfg, mesh, _ = bc_case(kind, types)
    for name in mesh.bcon:
        cfg.set(f'soln-bcs-{name}', 'quad-deg', qdeg)
    elemap = _elemap(cfg, mesh, kind == 'ns')
    nd = 2 if kind == 'euler' else 3
    m = np.array([0.3, -0.2, 0.45])[:nd]
    for name, side in mesh.bcon.items():
        si = SurfaceIntegrator(cfg, f'soln-bcs-{name}', elemap, side)
        # The boundary is the plane x_{nd-1} = 0 (outward normal -e) or 1
        # (+e), of unit area
        sgn = -1.0 if name.endswith('lo') else 1.0
        mf = area = pbar = 0.0
        solns = {}
        for et, e in elemap.items():
            pl = e.ploc_at_np('upts')                 # (nupts, nd, neles)
            u = np.zeros((e.nupts, e.nvars, e.neles))
            u[:, 0] = 1.0
            u[:, 1:nd + 1] = m[None, :, None]
            # p = 1 + 0.2 x_0 (linear along the boundary), E from it
            u[:, -1] = (1 + 0.2*pl[:, 0])/0.4 + 0.5*(m @ m)
            solns[et] = u
        for uf, w, n in si.interp(solns):
            mf += np.einsum('hij,hij', uf[1:-1], n*w[:, None])
            nm = np.sqrt(np.einsum('hij,hij->ij', n, n))*w[:, None]
            p = 0.4*(uf[-1] - 0.5*np.einsum('hij,hij->ij', uf[1:-1],
                                             uf[1:-1]))
            area += nm.sum()
            pbar += (p*nm).sum()
        assert abs(area - 1.0) < 1e-13
        assert abs(mf - sgn*m[-1]) < 1e-13
        assert abs(pbar/area - 1.1) < 1e-13


def test_surface_rule_selection():
    """The smallest Gauss rule exact for the requested degree, as the
    reference picks among its stored rules."""
    from pyfr_gb300.inifile import Inifile
    from pyfr_gb300.solvers.bccontrol import _face_rule
    cfg = Inifile()
    for qdeg, n in [(0, 1), (1, 1), (2, 2), (3, 2), (4, 3), (7, 4), (8, 5)]:
        cfg.set('soln-bcs-b', 'quad-deg', qdeg)
        pts, wts = _face_rule(cfg, 'soln-bcs-b', 'line')
        assert len(wts) == n
        pts, wts = _face_rule(cfg, 'soln-bcs-b', 'quad')
        assert len(wts) == n*n and abs(wts.sum() - 4) < 1e-14
    cfg.set('soln-bcs-b', 'quad-pts-line', 'gauss-legendre-lobatto')
    cfg.set('soln-bcs-b', 'quad-deg', 5)
    pts, wts = _face_rule(cfg, 'soln-bcs-b', 'line')
    assert len(wts) == 4 and abs(abs(pts).max() - 1) < 1e-15
