"""Meshes of several element types (hexahedra with prisms, prisms with
tetrahedra) through the CUDA path against the CPU oracle.

Plain FP64: relative max-norm tolerance 1e-10 on every conserved variable
of every element type, for the right-hand side on perturbed meshes (the
oracle given the reference's operators and geometry checked against the
reference's elements) and after RK45 steps.  The split-BF16 form must stay
within the relative L2 bound 1e-6 of the FP64 solution."""
import numpy as np
import pytest

from oracle.fr_oracle import rk45_step
from tests.test_oracle import MIXED_FPTS, MIXED_UPTS, mixed_disc

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
    spts = {et: g[f'{et}/spts'] for et in ('hex', 'pri', 'tet')
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


@pytest.mark.parametrize('case', ['hexpri_p3', 'pritet_p3'])
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


@pytest.mark.parametrize('kinds', ['hex-pri', 'pri-tet'])
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
        key = 'hex_p3_gauss-legendre' if et == 'hex' else f'{et}_p3_mixed'
        s = get_shape(et, 3, MIXED_UPTS[et], MIXED_FPTS)
        parts[et] = dict(ops=ops_from_golden(ops, key), basis=basis_of(s),
                         verts=verts)
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


@pytest.mark.parametrize('kinds', ['hex-pri', 'pri-tet'])
def test_mixed_mesh_chosen_form(built, kinds):
    """Split-BF16 operators (four products), FP32 fluxes, FP64 RK
    accumulation against the FP64 solution after ten steps."""
    from pyfr_gb300.cases import euler_mixed
    from pyfr_gb300.integrators import MixedRKIntegrator, RKVdH2Integrator
    from pyfr_gb300.solvers.system import EulerSystem

    cfg, mesh = euler_mixed(n=5, kinds=kinds, dt=2e-3)
    plain = RKVdH2Integrator(_backend(cfg), EulerSystem, mesh, cfg)
    plain.run_steps(10)

    cfg, mesh = euler_mixed(n=5, kinds=kinds, dt=2e-3, precision='single')
    cfg.set('backend-b200', 'mul-precision', 'bf16x3')
    cfg.set('backend-b200', 'split-products', '4')
    chosen = MixedRKIntegrator(_backend(cfg), EulerSystem, mesh, cfg)
    chosen.run_steps(10)
    for a, b in zip(chosen.soln, plain.soln):
        assert np.linalg.norm(a - b)/np.linalg.norm(b) <= 1e-6


@pytest.mark.parametrize('kinds', ['hex-pri', 'pri-tet'])
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
