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


@pytest.mark.parametrize('source', [False, True])
@pytest.mark.parametrize('case,n,steps', [('vortex', 8, 5), ('tgv', 3, 2)])
def test_reference_solver_on_b200(built, tmp_path, case, n, steps, source):
    """With ``source`` the case's [solver-plugin-source] terms go through
    PyFR's own source plugin (functions of position, solution and time;
    the oracle advances with the same stage times)."""
    if reference_tree() is None:
        pytest.skip('reference source tree not present')
    from oracle.fr_oracle import rk45_step_t
    from pyfr_gb300.cases import euler_vortex, ns_tgv
    from tests.oracle_util import SOURCES, disc_for_mesh, source_c_exprs

    out = tmp_path / 'soln.npz'
    r = subprocess.run([sys.executable, '-m', 'tests.refstack', '--case',
                        case, '--n', str(n), '--steps', str(steps), '--out',
                        str(out)] + (['--source'] if source else []),
                       cwd=ROOT, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    d = np.load(out)
    assert str(d['backend']) == 'B200Backend'
    assert int(d['nsteps']) == steps

    if case == 'vortex':
        cfg, mesh = euler_vortex(n=n, order=3, dt=1e-3)
        disc = disc_for_mesh(mesh, 3)
        c = cfg.items_as('constants', float)
        src = source_c_exprs(SOURCES[case], ['rho', 'rhou', 'rhov', 'E'],
                             c) if source else None
        rhs = lambda x, t: disc.rhs_euler(x, c, t=t, src=src)   # noqa: E731
    else:
        cfg, mesh = ns_tgv(n=n, order=3, dt=1e-3)
        disc = disc_for_mesh(mesh, 3, ns=True)
        c = cfg.items_as('constants', float) | \
            cfg.items_as('solver-interfaces', float)
        src = source_c_exprs(SOURCES[case],
                             ['rho', 'rhou', 'rhov', 'rhow', 'E'],
                             cfg.items_as('constants', float)) \
            if source else None
        rhs = lambda x, t: disc.rhs_ns(x, c, t=t, src=src)      # noqa: E731
    u, dt = d['u0'], float(d['dt'])
    for i in range(steps):
        u = rk45_step_t(rhs, u, i*dt, dt)
    err = max(np.abs(d['u1'][:, v] - u[:, v]).max()/np.abs(u[:, v]).max()
              for v in range(u.shape[1]))
    assert err < 1e-10, err


def test_reference_solver_single_fused(built, tmp_path):
    """PyFR's Euler system in single precision on the tensor-core applies,
    its divergence chain fused into one apply by the backend's fuser, five
    RK45 steps of the vortex against the oracle's FP64 steps: the FP32
    right-hand side is good to about 1e-4 of its scale, so the solution
    after five steps of 1e-3 to well under 1e-5."""
    import json
    if reference_tree() is None:
        pytest.skip('reference source tree not present')
    from oracle.fr_oracle import rk45_step
    from pyfr_gb300.cases import euler_vortex
    from tests.oracle_util import disc_for_mesh

    out = tmp_path / 'soln.npz'
    r = subprocess.run([sys.executable, '-m', 'tests.refstack', '--case',
                        'vortex', '--n', '8', '--steps', '5', '--single',
                        '--report', '--out', str(out)], cwd=ROOT,
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    graphs = json.loads(r.stdout.strip().splitlines()[-1])
    assert graphs[-1] == ['tflux', 'mul:bf16x3-cat']
    d = np.load(out)
    cfg, mesh = euler_vortex(n=8, order=3, dt=1e-3)
    disc = disc_for_mesh(mesh, 3)
    c = cfg.items_as('constants', float)
    u = d['u0'].astype(np.float64)
    for _ in range(5):
        u = rk45_step(lambda x: disc.rhs_euler(x, c), u, float(d['dt']))
    err = max(np.abs(d['u1'][:, v] - u[:, v]).max()/np.abs(u[:, v]).max()
              for v in range(u.shape[1]))
    assert err < 1e-5, err


BC_CASES = [('euler', ('sup-in-fa', 'sup-out-fn')),
            ('euler', ('char-riem-inv', 'slp-adia-wall')),
            ('ns', ('no-slp-isot-wall', 'sub-out-fp')),
            ('ns', ('sub-in-frv', 'sub-in-ftpttang')),
            ('ns', ('char-riem-inv', 'no-slp-adia-wall'))]


@pytest.mark.parametrize('kind,types', BC_CASES)
def test_reference_solver_boundaries(built, tmp_path, kind, types):
    """PyFR's own boundary interfaces (their values in the kernels'
    template arguments, pyfr/solvers/{euler,navstokes}/inters.py) on the
    b200 backend: three RK45 steps of a box bounded in one direction
    against the oracle's at 1e-10."""
    if reference_tree() is None:
        pytest.skip('reference source tree not present')
    from oracle.fr_oracle import rk45_step
    from tests.bc_cases import GAS, bc_case
    from tests.test_oracle import bc_disc

    out = tmp_path / 'soln.npz'
    r = subprocess.run([sys.executable, '-m', 'tests.refstack', '--case',
                        f'bc-{kind}:{",".join(types)}', '--steps', '3',
                        '--out', str(out)], cwd=ROOT, capture_output=True,
                       text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    d = np.load(out)
    _, _, specs = bc_case(kind, types)
    if kind == 'euler':
        disc, _ = bc_disc('quad', (4, 3), (True, False), specs)
        rhs = lambda x: disc.rhs_euler(x, GAS)           # noqa: E731
    else:
        disc, _ = bc_disc('hex', (2, 2, 3), (True, True, False), specs,
                          ns=True)
        rhs = lambda x: disc.rhs_ns(x, GAS)              # noqa: E731
    u = d['u0']
    for _ in range(3):
        u = rk45_step(rhs, u, float(d['dt']))
    err = max(np.abs(d['u1'][:, v] - u[:, v]).max()/np.abs(u[:, v]).max()
              for v in range(u.shape[1]))
    assert err < 1e-10, err


@pytest.mark.parametrize('kind,types', [
    ('euler', ('char-riem-inv-mass-flow', 'sup-out-fn')),
    ('ns', ('char-riem-inv-pressure', 'no-slp-adia-wall'))])
def test_reference_controlled_bcs(built, tmp_path, kind, types):
    """PyFR's own controlled boundaries (its host controller,
    pyfr/solvers/euler/inters.py:108-294, measuring the b200 solution and
    binding ic and im into the b200 kernels every right-hand side) against
    this package's controller on the same case: eight RK45 steps, with
    controller updates every three right-hand sides, agree at 1e-10."""
    if reference_tree() is None:
        pytest.skip('reference source tree not present')
    from pyfr_gb300.backend import B200Backend
    from pyfr_gb300.integrators import RKVdH2Integrator
    from pyfr_gb300.solvers.system import EulerSystem, NavierStokesSystem
    from tests.bc_cases import bc_case

    out = tmp_path / 'soln.npz'
    r = subprocess.run([sys.executable, '-m', 'tests.refstack', '--case',
                        f'bc-{kind}:{",".join(types)}', '--steps', '8',
                        '--out', str(out)], cwd=ROOT, capture_output=True,
                       text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    d = np.load(out)
    cfg, mesh, _ = bc_case(kind, types)
    cls = EulerSystem if kind == 'euler' else NavierStokesSystem
    intg = RKVdH2Integrator(B200Backend(cfg), cls, mesh, cfg)
    (u0,) = intg.soln
    assert np.abs(u0 - d['u0']).max() < 1e-14
    intg.run_steps(8)
    (u1,) = intg.soln
    (c,) = intg.system.controlled_bcs
    assert len(c.history) >= 10
    err = max(np.abs(d['u1'][:, v] - u1[:, v]).max()/np.abs(u1[:, v]).max()
              for v in range(u1.shape[1]))
    assert err < 1e-10, err
    # The controller moved the pressure: the run differs from one at the
    # initial pressure
    assert abs(c.interp_m) > 0


@pytest.mark.parametrize('kinds', ['hex-pyr-tet', 'pri-tet'])
def test_reference_solver_mixed_mesh(built, tmp_path, kinds):
    """PyFR's own Euler system and RK45 integrator on a mixed mesh
    (hexahedra, pyramids and tetrahedra: the reference's own pyramid shape
    and points) driven through the b200 backend, against the oracle with
    this package's operators: 1e-10 relative max-norm per type."""
    if reference_tree() is None:
        pytest.skip('reference source tree not present')
    from oracle.fr_oracle import MixedDiscretisation, rk45_step
    from pyfr_gb300.cases import euler_mixed
    from pyfr_gb300.shapes import get_shape
    from tests.oracle_util import basis_of, ops_from_shape
    from tests.test_oracle import MIXED_FPTS, MIXED_UPTS

    out = tmp_path / 'soln.npz'
    r = subprocess.run([sys.executable, '-m', 'tests.refstack', '--case',
                        f'mixed-{kinds}', '--n', '2', '--steps', '3',
                        '--out', str(out)],
                       cwd=ROOT, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    d = np.load(out)
    assert str(d['backend']) == 'B200Backend'
    ets = [str(e) for e in d['etypes']]

    cfg, mesh = euler_mixed(n=2, kinds=kinds, dt=1e-3)
    assert set(ets) == set(mesh.spts)
    parts = {}
    for et, verts in mesh.spts.items():
        s = get_shape(et, 3, MIXED_UPTS[et], MIXED_FPTS)
        parts[et] = dict(ops=ops_from_shape(s), basis=basis_of(s),
                         verts=verts)
    lhs, rhs = mesh.con
    disc = MixedDiscretisation(parts, zip(lhs.etypes, lhs.eidxs, lhs.fidxs),
                               zip(rhs.etypes, rhs.eidxs, rhs.fidxs),
                               periods=mesh.periods)
    c = dict(gamma=1.4)
    u = disc.pack({et: d[f'u0/{et}'] for et in ets})
    for _ in range(3):
        u = rk45_step(lambda x: disc.pack(disc.rhs_euler(disc.unpack(x, 5), c)),
                      u, float(d['dt']))
    ref = disc.unpack(u, 5)
    for et in ets:
        got = d[f'u1/{et}']
        err = max(np.abs(got[:, v] - ref[et][:, v]).max() /
                  np.abs(ref[et][:, v]).max() for v in range(5))
        assert err < 1e-10, (et, err)
