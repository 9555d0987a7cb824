"""Meshes of several element types (hexahedra with prisms, prisms with
tetrahedra, hexahedra with tetrahedra through pyramids) through the CUDA
path against the CPU oracle.

Plain FP64: relative max-norm tolerance 1e-10 on every conserved variable
of every element type, for the right-hand side on perturbed meshes (the
oracle given the reference's operators and geometry checked against the
reference's elements) and after RK45 steps.  The precision forms are held
to bounds set by their operands' significant bits."""
import numpy as np
import pytest

from oracle.fr_oracle import rk45_step
from tests.test_oracle import MIXED_FPTS, MIXED_UPTS, mixed_disc, mixed_key

pytestmark = pytest.mark.gpu

TOL = 1e-10


@pytest.fixture(scope='module')
def built():
    import __graft_entry__ as ge
    ge.build_library()


def _relerr(a, b):
    return np.abs(a - b).max()/max(np.abs(b).max(), 1e-300)


def _cfg(rsolver='rusanov'):
    from pyfr_gb300.inifile import Inifile
    cfg = Inifile()
    cfg.set('constants', 'gamma', 1.4)
    cfg.set('solver', 'order', 3)
    cfg.set('solver-interfaces', 'riemann-solver', rsolver)
    for et, r in MIXED_UPTS.items():
        cfg.set(f'solver-elements-{et}', 'soln-pts', r)
    for k, r in MIXED_FPTS.items():
        cfg.set(f'solver-interfaces-{k}', 'flux-pts', r)
    return cfg


def _golden_mesh(g):
    from pyfr_gb300.mesh import Mesh, Side
    spts = {et: g[f'{et}/spts'] for et in ('hex', 'pri', 'tet', 'pyr')
            if f'{et}/spts' in g}
    sides = [Side(s[:, 0], s[:, 1].astype(int), s[:, 2].astype(int))
             for s in (g['lhs'], g['rhs'])]
    return Mesh(ndims=3, spts=spts, con=tuple(sides),
                spts_curved={et: np.zeros(v.shape[1], bool)
                             for et, v in spts.items()},
                periods=(2.0,)*3)


def _backend(cfg):
    from pyfr_gb300.backend import B200Backend
    return B200Backend(cfg)


@pytest.mark.parametrize('case', ['hexpri_p3', 'pritet_p3', 'hexpyrtet_p3'])
@pytest.mark.parametrize('rsolver', ['rusanov', 'hllc'])
def test_euler_rhs_mixed_mesh(built, golden, case, rsolver):
    from pyfr_gb300.solvers.system import EulerSystem
    g = golden[f'geometry_{case}']
    mesh = _golden_mesh(g)
    cfg = _cfg(rsolver)
    ics = {et: g[f'{et}/ics'] for et in mesh.spts}
    s = EulerSystem(_backend(cfg), mesh, ics, 2, cfg)
    s.commit()
    s.rhs(0.0, 0, 1)
    got = dict(zip(s.ele_types, s.ele_scal_upts(1)))

    d, _ = mixed_disc(golden, case)
    ref = d.rhs_euler(ics, dict(gamma=1.4), rsolver)
    for et in mesh.spts:
        assert _relerr(got[et], ref[et]) < TOL, et


@pytest.mark.parametrize('kinds', ['hex-pri', 'pri-tet', 'hex-pyr-tet'])
def test_rk45_mixed_mesh(built, golden, kinds):
    """Three RK45 steps of the advected density wave, CUDA graphs on."""
    from oracle.fr_oracle import MixedDiscretisation
    from pyfr_gb300.cases import euler_mixed
    from pyfr_gb300.integrators import RKVdH2Integrator
    from pyfr_gb300.shapes import get_shape
    from pyfr_gb300.solvers.system import EulerSystem
    from tests.oracle_util import basis_of, ops_from_golden

    cfg, mesh = euler_mixed(n=4, kinds=kinds, dt=2e-3)
    intg = RKVdH2Integrator(_backend(cfg), EulerSystem, mesh, cfg)
    u0 = dict(zip(intg.system.ele_types, intg.soln))
    intg.run_steps(3)
    got = dict(zip(intg.system.ele_types, intg.soln))

    ops = golden['operators']
    parts = {}
    for et, verts in mesh.spts.items():
        s = get_shape(et, 3, MIXED_UPTS[et], MIXED_FPTS)
        parts[et] = dict(ops=ops_from_golden(ops, mixed_key(et)),
                         basis=basis_of(s), verts=verts)
    lhs, rhs = mesh.con
    d = MixedDiscretisation(parts, zip(lhs.etypes, lhs.eidxs, lhs.fidxs),
                            zip(rhs.etypes, rhs.eidxs, rhs.fidxs),
                            periods=mesh.periods)
    c = dict(gamma=1.4)
    u = d.pack(u0)
    for _ in range(3):
        u = rk45_step(lambda x: d.pack(d.rhs_euler(d.unpack(x, 5), c)),
                      u, 2e-3)
    ref = d.unpack(u, 5)
    for et in mesh.spts:
        assert _relerr(got[et], ref[et]) < TOL, et


@pytest.mark.parametrize('kinds', ['hex-pri', 'pri-tet', 'hex-pyr-tet'])
def test_mixed_mesh_precision_forms(built, kinds):
    """The precision forms (FP32 fluxes, FP64 RK accumulation) against the
    FP64 solution after ten steps, without the reference-state transform
    (``reference-shift = none``; with it the mean flow leaves the fluxes,
    test_gpu_chosen.py).  This flow then carries O(1) mean fluxes, so the
    operator's representation error times the mean flux shows directly: split-BF16 operands carry 17
    significant bits (1.6e-6 measured, bound 1e-5), single TF32 operands
    11 bits (2.1e-4 measured on prisms, bound 5e-4); plain FP32
    arithmetic is at 1.5e-7.  The operator in three BF16 terms (five
    products) removes the operator's share (3.9e-7 to 4.9e-7 measured,
    bound 1e-6)."""
    from pyfr_gb300.cases import euler_mixed
    from pyfr_gb300.integrators import MixedRKIntegrator, RKVdH2Integrator
    from pyfr_gb300.solvers.system import EulerSystem

    def run(precision, mul=None, icls=RKVdH2Integrator, nprod='4'):
        cfg, mesh = euler_mixed(n=5, kinds=kinds, dt=2e-3,
                                precision=precision)
        cfg.set('backend-b200', 'reference-shift', 'none')
        if mul:
            cfg.set('backend-b200', 'mul-precision', mul)
            if mul == 'bf16x3':
                cfg.set('backend-b200', 'split-products', nprod)
        intg = icls(_backend(cfg), EulerSystem, mesh, cfg)
        intg.run_steps(10)
        return [np.asarray(u, dtype=np.float64) for u in intg.soln]

    def l2(a, b):
        return np.linalg.norm(a - b)/np.linalg.norm(b)

    plain = run('double')
    fp32 = run('single')
    bf16 = run('single', 'bf16x3', MixedRKIntegrator)
    bf16t3 = run('single', 'bf16x3', MixedRKIntegrator, '5')
    tf32 = run('single', 'tf32', MixedRKIntegrator)
    for b, b5, f, t, p in zip(bf16, bf16t3, fp32, tf32, plain):
        e32, eb, e5, et = l2(f, p), l2(b, p), l2(b5, p), l2(t, p)
        assert eb <= 1e-5 and eb <= et, (eb, et, e32)
        assert et <= 5e-4, (et, e32)
        assert e5 <= 1e-6, (e5, eb, e32)


@pytest.mark.parametrize('kinds', ['hex-pri', 'pri-tet', 'hex-pyr-tet'])
def test_mixed_mesh_density_wave_accuracy(built, kinds):
    """The advected density wave stays close to its exact translation
    (a discretisation check, independent of the oracle).  With six cells
    per direction the oracle's own errors after 40 steps are 7e-4
    (hexes), 3e-3 to 6e-3 (prisms) and 1.2e-2 (tetrahedra), converging at
    about fourth order under refinement."""
    from pyfr_gb300.cases import density_wave_exact, euler_mixed
    from pyfr_gb300.integrators import RKVdH2Integrator
    from pyfr_gb300.solvers.system import EulerSystem

    cfg, mesh = euler_mixed(n=6, kinds=kinds, dt=5e-3)
    intg = RKVdH2Integrator(_backend(cfg), EulerSystem, mesh, cfg)
    intg.run_steps(40)
    for u, ploc in zip(intg.soln, intg.system.ele_ploc_upts):
        rho = density_wave_exact(ploc[:, 0], ploc[:, 1], ploc[:, 2],
                                 intg.tcurr, cfg)
        assert np.abs(u[:, 0] - rho).max() < 2e-2


@pytest.mark.parametrize('case', ['hexpri_p3', 'pritet_p3', 'hexpyrtet_p3'])
@pytest.mark.parametrize('beta', [0.5, 0.0])
def test_ns_rhs_mixed_mesh(built, golden, case, beta):
    """Navier-Stokes on the perturbed mixed meshes (gradient operators of
    prisms and tetrahedra included) against the multi-type oracle."""
    from oracle.fr_oracle import MixedDiscretisation
    from pyfr_gb300.shapes import get_shape
    from pyfr_gb300.solvers.system import NavierStokesSystem
    from tests.oracle_util import basis_of, ops_from_golden
    g = golden[f'geometry_{case}']
    mesh = _golden_mesh(g)
    cfg = _cfg('rusanov')
    gas = dict(gamma=1.4, mu=0.03, Pr=0.72, **{'ldg-beta': beta,
                                              'ldg-tau': 0.1})
    for k in ('mu', 'Pr'):
        cfg.set('constants', k, gas[k])
    cfg.set('solver-interfaces', 'ldg-beta', beta)
    cfg.set('solver-interfaces', 'ldg-tau', 0.1)
    ics = {et: g[f'{et}/ics'] for et in mesh.spts}
    s = NavierStokesSystem(_backend(cfg), mesh, ics, 2, cfg)
    s.commit()
    s.rhs(0.0, 0, 1)
    got = dict(zip(s.ele_types, s.ele_scal_upts(1)))

    ops = golden['operators']
    parts = {}
    for et in mesh.spts:
        sh = get_shape(et, 3, MIXED_UPTS[et], MIXED_FPTS)
        parts[et] = dict(ops=ops_from_golden(ops, mixed_key(et), True),
                         basis=basis_of(sh), verts=mesh.spts[et])
    d = MixedDiscretisation(parts, g['lhs'], g['rhs'], periods=(2.0,)*3)
    ref = d.rhs_ns(ics, gas)
    for et in mesh.spts:
        assert _relerr(got[et], ref[et]) < TOL, et


@pytest.mark.parametrize('system', ['euler', 'navier-stokes'])
def test_triangle_mesh_rhs(built, system):
    """2-D triangles (each cell of a periodic square cut in two)."""
    from oracle.fr_oracle import MixedDiscretisation
    from pyfr_gb300.inifile import Inifile
    from pyfr_gb300.mesh import tri_box
    from pyfr_gb300.shapes import get_shape
    from pyfr_gb300.solvers.system import EulerSystem, NavierStokesSystem
    from tests.oracle_util import basis_of, ops_from_shape
    mesh = tri_box(5, -1.0, 1.0)
    cfg = Inifile()
    gas = dict(gamma=1.4, mu=0.02, Pr=0.72, **{'ldg-beta': 0.5,
                                              'ldg-tau': 0.1})
    for k in ('gamma', 'mu', 'Pr'):
        cfg.set('constants', k, gas[k])
    cfg.set('solver', 'order', 3)
    cfg.set('solver-interfaces', 'riemann-solver', 'rusanov')
    cfg.set('solver-interfaces', 'ldg-beta', 0.5)
    cfg.set('solver-interfaces', 'ldg-tau', 0.1)
    cfg.set('soln-ics', 'rho', '1 + 0.2*sin(pi*x)*cos(pi*y)')
    cfg.set('soln-ics', 'u', '0.4 + 0.1*y')
    cfg.set('soln-ics', 'v', '-0.2 + 0.1*sin(pi*x)')
    cfg.set('soln-ics', 'p', '1 + 0.1*cos(pi*x)')
    ns = system == 'navier-stokes'
    scls = NavierStokesSystem if ns else EulerSystem
    s = scls(_backend(cfg), mesh, None, 2, cfg)
    s.commit()
    s.rhs(0.0, 0, 1)
    (u,), (r,) = s.ele_scal_upts(0), s.ele_scal_upts(1)

    sh = get_shape('tri', 3, 'alpha-opt', 'gauss-legendre')
    lhs, rhs = mesh.con
    d = MixedDiscretisation(
        {'tri': dict(ops=ops_from_shape(sh, ns), basis=basis_of(sh),
                     verts=mesh.spts['tri'])},
        zip(lhs.etypes, lhs.eidxs, lhs.fidxs),
        zip(rhs.etypes, rhs.eidxs, rhs.fidxs), periods=mesh.periods)
    ref = (d.rhs_ns if ns else d.rhs_euler)({'tri': u}, gas)['tri']
    assert _relerr(r, ref) < TOL


@pytest.mark.parametrize('kinds', ['hex-pri', 'hex-pyr-tet'])
def test_mixed_mesh_chosen_form_shifted(built, kinds):
    """The chosen form (split BF16 with the three-term operator) on the
    moving density wave with the reference-state transform of its mean flow
    (the default): within 1e-6 of FP64 after ten steps, and at most half
    the error of the same form on unshifted inputs."""
    from pyfr_gb300.cases import euler_mixed
    from pyfr_gb300.integrators import MixedRKIntegrator, RKVdH2Integrator
    from pyfr_gb300.solvers.system import EulerSystem

    def run(precision, shift='auto'):
        cfg, mesh = euler_mixed(n=5, kinds=kinds, dt=2e-3,
                                precision=precision)
        icls = RKVdH2Integrator
        if precision == 'single':
            cfg.set('backend-b200', 'mul-precision', 'bf16x3')
            cfg.set('backend-b200', 'split-products', 5)
            cfg.set('backend-b200', 'reference-shift', shift)
            icls = MixedRKIntegrator
        intg = icls(_backend(cfg), EulerSystem, mesh, cfg)
        if precision == 'single':
            assert (intg.uref is not None) == (shift == 'auto')
        intg.run_steps(10)
        return [np.asarray(u, dtype=np.float64) for u in intg.soln]

    plain = run('double')
    shifted, unshifted = run('single'), run('single', 'none')
    for a, b, p in zip(shifted, unshifted, plain):
        es = np.linalg.norm(a - p)/np.linalg.norm(p)
        eu = np.linalg.norm(b - p)/np.linalg.norm(p)
        assert es <= 1e-6 and es <= 0.5*eu, (es, eu)
