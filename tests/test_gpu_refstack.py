"""The drop-in boundary end to end: PyFR's own EulerSystem /
NavierStokesSystem and RK45 integrator, from the reference's source tree,
selected and driven through ``get_backend('b200', cfg)`` and
``get_solver`` (``tests/refstack.py``), advance the 2-D vortex and the
Taylor-Green vortex on the GPU; the result equals the oracle's RK45 steps
from the same initial state within 1e-10 (relative max-norm per conserved
variable)."""
import subprocess
import sys

import numpy as np
import pytest

from tests.refstack import ROOT, reference_tree

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def built():
    import __graft_entry__ as ge
    ge.build_library()


@pytest.mark.parametrize('case,n,steps', [('vortex', 8, 5), ('tgv', 3, 2)])
def test_reference_solver_on_b200(built, tmp_path, case, n, steps):
    if reference_tree() is None:
        pytest.skip('reference source tree not present')
    from oracle.fr_oracle import rk45_step
    from pyfr_gb300.cases import euler_vortex, ns_tgv
    from tests.oracle_util import disc_for_mesh

    out = tmp_path / 'soln.npz'
    r = subprocess.run([sys.executable, '-m', 'tests.refstack', '--case',
                        case, '--n', str(n), '--steps', str(steps), '--out',
                        str(out)], cwd=ROOT, capture_output=True, text=True,
                       timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    d = np.load(out)
    assert str(d['backend']) == 'B200Backend'
    assert int(d['nsteps']) == steps

    if case == 'vortex':
        cfg, mesh = euler_vortex(n=n, order=3, dt=1e-3)
        disc = disc_for_mesh(mesh, 3)
        c = cfg.items_as('constants', float)
        rhs = lambda x: disc.rhs_euler(x, c)           # noqa: E731
    else:
        cfg, mesh = ns_tgv(n=n, order=3, dt=1e-3)
        disc = disc_for_mesh(mesh, 3, ns=True)
        c = cfg.items_as('constants', float) | \
            cfg.items_as('solver-interfaces', float)
        rhs = lambda x: disc.rhs_ns(x, c)              # noqa: E731
    u = d['u0']
    for _ in range(steps):
        u = rk45_step(rhs, u, float(d['dt']))
    err = max(np.abs(d['u1'][:, v] - u[:, v]).max()/np.abs(u[:, v]).max()
              for v in range(u.shape[1]))
    assert err < 1e-10, err
