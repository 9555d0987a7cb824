"""Runs on meshes read from files, solution output and restarts
(pyfr/readers/native.py, pyfr/plugins/writer.py, the restart path of
pyfr/integrators/base.py:48-65).

* the right-hand side on a Gmsh-imported box equals the one on the same
  box generated in memory (relative max-norm 1e-12; the interfaces come in
  another order);
* a run that writes its solution every two steps and is restarted from the
  middle output ends bit-identical to the uninterrupted run, with the
  fixed-step and the PI controllers and with the mixed-precision form."""
import numpy as np
import pytest

from tests.gmsh_util import box_msh

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def built():
    import __graft_entry__ as ge
    ge.build_library()


def _backend(cfg):
    from pyfr_gb300.backend import B200Backend
    return B200Backend(cfg)


@pytest.mark.parametrize('system', ['euler', 'navier-stokes'])
def test_rhs_on_imported_mesh(built, tmp_path, system):
    """The file's interfaces take their left side by the reference's rule
    (the face with the smaller codec key), the generated box by its own, so
    the comparison uses fluxes that do not favour a side: Rusanov, and for
    Navier-Stokes an LDG common solution with beta = 0."""
    from pyfr_gb300.gmsh import import_mesh
    from pyfr_gb300.mesh import box
    from pyfr_gb300.native import read_mesh
    from pyfr_gb300.solvers.system import EulerSystem, NavierStokesSystem
    from tests.test_gpu_bcs import FREE, _cfg

    n, per = (3, 2, 2), (True, False, True)
    import_mesh(box_msh(n, per, '4.1'), tmp_path / 'b.pyfrm')
    mfile = read_mesh(tmp_path / 'b.pyfrm')
    mgen = box('hex', n, 0.0, 1.0, per)
    specs = {'ylo': dict(type='no-slp-isot-wall', cpTw=3.2, **FREE),
             'yhi': dict(type='char-riem-inv', **FREE)}

    ns = system == 'navier-stokes'
    scls = NavierStokesSystem if ns else EulerSystem
    if not ns:
        specs['ylo'] = dict(type='slp-adia-wall')
    out = []
    for m in (mfile, mgen):
        cfg = _cfg(3, specs, ns=ns)
        cfg.set('solver-interfaces', 'ldg-beta', '0.0')
        s = scls(_backend(cfg), m, None, 2, cfg)
        s.commit()
        s.rhs(0.0, 0, 1)
        (r,) = s.ele_scal_upts(1)
        out.append(r)
    a, b = out
    assert np.abs(a - b).max()/np.abs(b).max() < 1e-12


def _vortex(tmp_path, controller, precision='double'):
    from pyfr_gb300.cases import euler_vortex
    from pyfr_gb300.native import read_mesh, save_mesh

    cfg, mesh = euler_vortex(n=8, order=3, dt=2e-3, precision=precision)
    save_mesh(tmp_path / 'v.pyfrm', mesh)
    sect = 'solver-time-integrator'
    if controller == 'pi':
        cfg.set(sect, 'controller', 'pi')
        cfg.set(sect, 'rtol', '1e-6')
        cfg.set(sect, 'atol', '1e-6')
    w = 'soln-plugin-writer'
    cfg.set(w, 'dt-out', '0.004')
    cfg.set(w, 'basedir', str(tmp_path))
    cfg.set(w, 'basename', 'vortex-{n:03d}')
    if precision == 'single':
        cfg.set('backend-b200', 'mul-precision', 'bf16x3')
        cfg.set('backend-b200', 'split-products', '5')
    return cfg, read_mesh(tmp_path / 'v.pyfrm')


@pytest.mark.parametrize('controller,form', [('none', 'plain'),
                                             ('pi', 'plain'),
                                             ('none', 'mixed'),
                                             ('none', 'mixed-shift')])
def test_restart_bit_identical(built, tmp_path, controller, form):
    """A restart from a written solution continues as the uninterrupted
    run: bit for bit, except with the mixed form's reference-state
    transform, where the run's reference state is restored from the file
    but the solution passes through u = q + u_ref and back, which rounds
    at the FP64 level (1e-13)."""
    from pyfr_gb300.integrators import MixedRKIntegrator, RKVdH2Integrator
    from pyfr_gb300.native import read_soln
    from pyfr_gb300.plugins import WriterPlugin
    from pyfr_gb300.solvers.system import EulerSystem

    icls = MixedRKIntegrator if form.startswith('mixed') else \
        RKVdH2Integrator
    prec = 'single' if form.startswith('mixed') else 'double'
    cfg, mesh = _vortex(tmp_path, controller, prec)
    if form == 'mixed':
        cfg.set('backend-b200', 'reference-shift', 'none')

    intg = icls(_backend(cfg), EulerSystem, mesh, cfg)
    wr = WriterPlugin(intg)
    intg.add_plugin(wr)
    intg.advance_to(0.012)
    (ufull,) = intg.soln
    names = [p.name for p in wr.files]
    assert names[:4] == ['vortex-000.pyfrs', 'vortex-001.pyfrs',
                         'vortex-002.pyfrs', 'vortex-003.pyfrs']
    assert len(names) == 4

    # Restart from the output at t = 0.004
    soln = read_soln(wr.files[1], mesh)
    assert soln.stats.getfloat('solver-time-integrator', 'tcurr') == \
        pytest.approx(0.004, abs=1e-15)
    if controller == 'pi':
        assert 'intg/ctrl' in soln.state
    cfg2 = soln.config
    cfg2.set('soln-plugin-writer', 'basename', 'restart-{n:03d}')
    intg2 = icls(_backend(cfg2), EulerSystem, mesh, cfg2, soln)
    assert intg2.isrestart and intg2.tcurr == \
        soln.stats.getfloat('solver-time-integrator', 'tcurr')
    wr2 = WriterPlugin(intg2)
    intg2.add_plugin(wr2)
    assert wr2.files == []                  # no initial output on restart
    if form == 'mixed-shift':
        assert 'intg/uref' in soln.state
        assert np.array_equal(intg2.uref, intg.uref)
    intg2.advance_to(0.012)
    (urest,) = intg2.soln
    if form == 'mixed-shift':
        assert np.abs(urest - ufull).max() <= 1e-13*np.abs(ufull).max()
    else:
        assert np.array_equal(urest, ufull)
    assert [p.name for p in wr2.files] == ['restart-000.pyfrs',
                                           'restart-001.pyfrs']

    s2 = read_soln(wr2.files[-1], mesh)
    if form != 'mixed-shift':
        assert np.array_equal(s2.data['quad'], ufull)
    assert sorted(s2.prevcfgs) == ['config-0', 'config-1']


def test_writer_gradients(built, tmp_path):
    """write-gradients: the physical gradients of the written solution
    (the system's gradient pass, pyfr/plugins/writer.py:27-33,113-116)
    against the oracle's corrected gradients of the same solution."""
    from pyfr_gb300.backend import B200Backend
    from pyfr_gb300.cases import ns_tgv
    from pyfr_gb300.integrators import RKVdH2Integrator
    from pyfr_gb300.native import read_soln, save_mesh, read_mesh
    from pyfr_gb300.plugins import WriterPlugin
    from pyfr_gb300.solvers.system import NavierStokesSystem
    from tests.oracle_util import disc_for_mesh

    cfg, mesh = ns_tgv(n=3, order=3, dt=5e-4)
    w = 'soln-plugin-writer'
    cfg.set(w, 'dt-out', '0.001')
    cfg.set(w, 'basedir', str(tmp_path))
    cfg.set(w, 'basename', 'tgv-{t:.3f}')
    cfg.set(w, 'write-gradients', 'true')
    save_mesh(tmp_path / 't.pyfrm', mesh)
    fmesh = read_mesh(tmp_path / 't.pyfrm')
    intg = RKVdH2Integrator(B200Backend(cfg), NavierStokesSystem, fmesh, cfg)
    wr = WriterPlugin(intg)
    intg.add_plugin(wr)
    intg.advance_to(0.001)
    s = read_soln(wr.files[-1], fmesh)
    u = s.data['hex']
    # (the oracle on the mesh read from the file: its interfaces take the
    # left side by the file's rule, which the LDG common solution sees)
    fmesh.periods = mesh.periods
    d = disc_for_mesh(fmesh, 3, ns=True)
    c = cfg.items_as('constants', float) | cfg.items_as('solver-interfaces',
                                                       float)
    gout = []
    d.rhs_ns(u, c, grads_out=gout)
    g = s.grad_data['hex']
    assert g.shape == gout[0].shape
    assert np.abs(g - gout[0]).max()/np.abs(gout[0]).max() < 1e-10
