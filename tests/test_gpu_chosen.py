"""The chosen precision form: FP32 right-hand side (operators and fluxes),
FP64 solution accumulation.  Its solution must stay within a relative L2
error of 1e-6 of the FP64 oracle; single RHS evaluations are checked at
FP32 accuracy (relative max-norm 1e-4 of the RHS scale)."""
import numpy as np
import pytest

from oracle.fr_oracle import rk45_step
from tests.oracle_util import disc_for_mesh

pytestmark = pytest.mark.gpu

L2_TOL = 1e-6


def _l2rel(a, b):
    return np.linalg.norm((a - b).ravel())/np.linalg.norm(b.ravel())


@pytest.fixture(scope='module')
def built():
    import __graft_entry__ as ge
    ge.build_library()


@pytest.mark.parametrize('key', ['hex_p3_gauss-legendre', 'quad_p3_gauss-legendre',
                                 'hex_p2_gauss-legendre',
                                 'hex_p4_gauss-legendre'])
@pytest.mark.parametrize('opname', ['m0', 'M132', 'm3', 'M460', 'm6'])
@pytest.mark.parametrize('prec', ['bf16x3-3', 'bf16x3-4', 'tf32'])
def test_mul_tensor_cores(built, golden, key, opname, prec):
    """tcgen05 operator apply against an FP64 product.  Split BF16 with
    three products is bounded by ~2^-16 sum|a||b| (bound 1e-4), with four
    by ~2^-17 (bound 5e-5); TF32 rounds both operands to 11 significant
    bits, ~2^-10 sum|a||b| (bound 2e-3).  Operators that do not fit one
    handle (p = 4: 375 rows, or K = 375) run as row and K pieces."""
    from pyfr_gb300.backend import B200Backend
    from pyfr_gb300.inifile import Inifile
    a = golden['operators'][f'{key}/{opname}']
    cfg = Inifile()
    cfg.set('backend', 'precision', 'single')
    mp, _, nprod = prec.partition('-')
    cfg.set('backend-b200', 'mul-precision', mp)
    if nprod:
        cfg.set('backend-b200', 'split-products', nprod)
    rel = {'bf16x3-3': 1e-4, 'bf16x3-4': 5e-5, 'tf32': 2e-3}[prec]
    be = B200Backend(cfg)
    rng = np.random.default_rng(7)
    for nvars, neles in [(5, 77), (4, 1000)]:
        b = rng.normal(size=(a.shape[1], nvars, neles))
        c0 = rng.normal(size=(a.shape[0], nvars, neles))
        A = be.const_matrix(a)
        B = be.matrix(b.shape, b, tags={'align'})
        C = be.matrix(c0.shape, c0, tags={'align'})
        be.commit()
        bound = rel*np.einsum('mk,kve->mve', np.abs(a), np.abs(b)) + 1e-6
        for alpha, beta in [(1.0, 0.0), (1.0, 1.0), (-0.5, 1.0), (2.0, 0.25)]:
            C.set(c0)
            k = be.kernel('mul', A, B, out=C, alpha=alpha, beta=beta)
            # The tensor-core epilogue stores or adds; other beta fall back
            assert k.meta['impl'] == (mp if beta in (0.0, 1.0) else 'csr')
            be.run_kernels([k], wait=True)
            ref = alpha*np.einsum('mk,kve->mve', a, b.astype(np.float32)) + \
                beta*c0.astype(np.float32)
            assert np.all(np.abs(C.get() - ref) <= abs(alpha)*bound +
                          1e-6*np.abs(ref))


def _bf16_pair_exact(x):
    """Values with at most 16 significant bits (exact as BF16 hi + lo)."""
    x = np.asarray(x, dtype=np.float32)
    u = x.view(np.uint32) & np.uint32(0xffff8000)
    return u.view(np.float32).astype(np.float64)


@pytest.mark.parametrize('key', ['hex_p3_gauss-legendre', 'quad_p3_gauss-legendre',
                                 'pri_p3_mixed', 'tet_p3_mixed'])
@pytest.mark.parametrize('opname', ['m0', 'M132', 'm3', 'M460', 'm6'])
def test_mul_three_term_operator(built, golden, key, opname):
    """Five products (operator in three BF16 terms): on data whose split
    is exact, a large uniform offset included, the only error left is the
    FP32 accumulation (bound 2e-6 sum|a||b|, where the two-term operator's
    own error is ~2^-17 sum|a||b|)."""
    from pyfr_gb300.backend import B200Backend
    from pyfr_gb300.inifile import Inifile
    a = golden['operators'][f'{key}/{opname}']
    cfg = Inifile()
    cfg.set('backend', 'precision', 'single')
    cfg.set('backend-b200', 'mul-precision', 'bf16x3')
    cfg.set('backend-b200', 'split-products', '5')
    be = B200Backend(cfg)
    rng = np.random.default_rng(9)
    b = _bf16_pair_exact(3.0 + 0.1*rng.normal(size=(a.shape[1], 5, 333)))
    A = be.const_matrix(a)
    B = be.matrix(b.shape, b, tags={'align'})
    C = be.matrix((a.shape[0], 5, 333), tags={'align'})
    be.commit()
    k = be.kernel('mul', A, B, out=C)
    assert k.meta['products'] == 5
    be.run_kernels([k], wait=True)
    ref = np.einsum('mk,kve->mve', a, b)
    bound = 2e-6*np.einsum('mk,kve->mve', np.abs(a), np.abs(b)) + 1e-7
    assert np.all(np.abs(C.get() - ref) <= bound)


@pytest.mark.parametrize('neles,order,nprod', [(77, 3, '3'), (1000, 3, '3'),
                                              (333, 4, '5'), (333, 3, '5')])
def test_mul_bf16x3_cat_rowscale(built, golden, neles, order, nprod):
    """Fused apply out = alpha*S*(A1@B1 + A2@B2) (+ out): the divergence,
    correction and negdivconf of the reference in one kernel (at p = 4 in
    K pieces, each scaled and the later ones added)."""
    from pyfr_gb300.backend import B200Backend
    from pyfr_gb300.inifile import Inifile
    ops = golden['operators']
    a1 = ops[f'hex_p{order}_gauss-legendre/M132']
    a2 = ops[f'hex_p{order}_gauss-legendre/m3']
    cfg = Inifile()
    cfg.set('backend', 'precision', 'single')
    cfg.set('backend-b200', 'mul-precision', 'bf16x3')
    cfg.set('backend-b200', 'split-products', nprod)
    be = B200Backend(cfg)
    rng = np.random.default_rng(11)
    nv = 5
    b1 = rng.normal(size=(a1.shape[1], nv, neles))
    b2 = rng.normal(size=(a2.shape[1], nv, neles))
    c0 = rng.normal(size=(a1.shape[0], nv, neles))
    sc = rng.uniform(0.5, 2.0, size=(a1.shape[0], neles))
    A1, A2 = be.const_matrix(a1), be.const_matrix(a2)
    B1 = be.matrix(b1.shape, b1, tags={'align'})
    B2 = be.matrix(b2.shape, b2, tags={'align'})
    C_ = be.matrix(c0.shape, c0, tags={'align'})
    S = be.matrix(sc.shape, sc, tags={'align'})
    be.commit()
    b1f, b2f = b1.astype(np.float32), b2.astype(np.float32)
    prod = np.einsum('mk,kve->mve', a1, b1f) + np.einsum('mk,kve->mve', a2, b2f)
    bound = 1e-4*(np.einsum('mk,kve->mve', np.abs(a1), np.abs(b1f)) +
                  np.einsum('mk,kve->mve', np.abs(a2), np.abs(b2f))) + 1e-6
    for alpha, beta, rs in [(1.0, 0.0, None), (-1.0, 0.0, S), (0.5, 1.0, S)]:
        C_.set(c0)
        k = be.kernel('mul_cat', A1, B1, A2, B2, out=C_, alpha=alpha,
                      beta=beta, rowscale=rs)
        assert k.meta['impl'] == 'bf16x3-cat'
        be.run_kernels([k], wait=True)
        f = alpha*(sc[:, None, :] if rs is not None else 1.0)
        ref = f*prod + beta*c0.astype(np.float32)
        assert np.all(np.abs(C_.get() - ref) <= np.abs(f)*bound +
                      1e-6*np.abs(ref))


@pytest.mark.parametrize('op', ['hex_p3_gauss-legendre/m0',
                                'hex_p4_gauss-legendre/m0',
                                'hex_p4_gauss-legendre/m6'])
def test_mul_bf16x3_batched(built, golden, op):
    """ndims products of one operator as one launch over row slices."""
    from pyfr_gb300.backend import B200Backend
    from pyfr_gb300.inifile import Inifile
    a = golden['operators'][op]
    cfg = Inifile()
    cfg.set('backend', 'precision', 'single')
    cfg.set('backend-b200', 'mul-precision', 'bf16x3')
    be = B200Backend(cfg)
    rng = np.random.default_rng(12)
    nb, nv, neles = 3, 5, 333
    b = rng.normal(size=(nb, a.shape[1], nv, neles))
    B = be.matrix(b.shape, b, tags={'align'})
    C_ = be.matrix((nb, a.shape[0], nv, neles), tags={'align'})
    A = be.const_matrix(a)
    be.commit()
    k = be.kernel('mul_batched', A, B, C_, nbatch=nb)
    be.run_kernels([k], wait=True)
    bf = b.astype(np.float32)
    ref = np.einsum('mk,zkve->zmve', a, bf)
    bound = 1e-4*np.einsum('mk,zkve->zmve', np.abs(a), np.abs(bf)) + 1e-6
    assert np.all(np.abs(C_.get() - ref) <= bound)


def test_fused_ns_rhs_matches_oracle(built):
    """The fused graph (corrected gradient, face gradients, and divergence
    with negdivconf as three fused applies) against the unfused graph, both
    split-BF16 on the reference-state transform of the TGV.  Split-BF16
    products carry about 2^-16 sum|a||b| of error, and the divergence
    operator's rows sum to tens, so the RHS error is about 1e-3 of its
    size (bound 3e-3); fusing must not make it worse (it skips two FP32
    roundings of partial results)."""
    from pyfr_gb300.backend import B200Backend
    from pyfr_gb300.cases import ns_tgv
    from pyfr_gb300.solvers.system import NavierStokesSystem
    out = {}
    for fuse in ('true', 'false'):
        cfg, mesh = ns_tgv(n=5, order=3, precision='single')
        cfg.set('backend-b200', 'mul-precision', 'bf16x3')
        cfg.set('backend-b200', 'fuse-operators', fuse)
        gamma = cfg.getfloat('constants', 'gamma')
        be = B200Backend(cfg)
        assert be.fuse_operators == (fuse == 'true')
        s = NavierStokesSystem(be, mesh, None, 2, cfg)
        (eles,) = s.ele_map.values()
        u = eles.set_ics_from_cfg()
        rho_ref, p_ref = 1.0, cfg.getfloat('constants', 'p0')
        hs = gamma/(gamma - 1)*p_ref/rho_ref
        be.ref_state = (rho_ref, p_ref)
        s.commit()
        q = u - np.array([rho_ref, 0, 0, 0, p_ref/(gamma - 1)])[None, :, None]
        q[:, -1] -= hs*q[:, 0]
        s.ele_banks[0][0].set(q.astype(np.float32))
        s.rhs(0.0, 0, 1)
        (out[fuse],) = s.ele_scal_upts(1)

    d = disc_for_mesh(mesh, 3, ns=True)
    c = cfg.items_as('constants', float) | cfg.items_as('solver-interfaces',
                                                       float)
    ref = d.rhs_ns(u, c)
    ref[:, -1] -= hs*ref[:, 0]
    err = {f: np.abs(out[f] - ref).max()/np.abs(ref).max() for f in out}
    assert err['false'] <= 3e-3
    assert err['true'] <= 1.5*err['false']


def test_fp32_ns_rhs(built):
    """The TGV fluxes carry the mean pressure p0 = 1/(gamma Ma^2) ~ 71
    while the RHS is O(1): FP32 rounding of the fluxes (relative 6e-8 of
    p0) is amplified by the divergence and lift operators, so the RHS error
    is bounded relative to p0/h, not to the RHS itself.  A numpy emulation
    of the same arithmetic in float32 gives 6e-5 p0/h on this case; the
    bound is 1e-4 p0/h."""
    from pyfr_gb300.backend import B200Backend
    from pyfr_gb300.cases import ns_tgv
    from pyfr_gb300.solvers.system import NavierStokesSystem
    cfg, mesh = ns_tgv(n=5, order=3, precision='single')
    be = B200Backend(cfg)
    s = NavierStokesSystem(be, mesh, None, 2, cfg)
    s.commit()
    s.rhs(0.0, 0, 1)
    (u,), (r,) = s.ele_scal_upts(0), s.ele_scal_upts(1)
    assert r.dtype == np.float32

    d = disc_for_mesh(mesh, 3, ns=True)
    c = cfg.items_as('constants', float) | cfg.items_as('solver-interfaces',
                                                       float)
    ref = d.rhs_ns(u.astype(np.float64), c)
    h = 2*np.pi/5
    assert np.abs(r - ref).max() <= 1e-4*c['p0']/h


def test_fp32_ns_rhs_reference_shift(built):
    """With the reference-state transform the FP32 input is
    q = T(u - u_ref) (energy replaced by dE - h_ref*drho) and the kernels
    return T times the right-hand side: no flux carries the mean pressure
    or enthalpy any more, so the error is bounded relative to the RHS
    itself (1e-4 on every variable)."""
    from pyfr_gb300.backend import B200Backend
    from pyfr_gb300.cases import ns_tgv
    from pyfr_gb300.solvers.system import NavierStokesSystem
    cfg, mesh = ns_tgv(n=5, order=3, precision='single')
    gamma = cfg.getfloat('constants', 'gamma')
    be = B200Backend(cfg)
    s = NavierStokesSystem(be, mesh, None, 2, cfg)
    (eles,) = s.ele_map.values()
    u = eles.set_ics_from_cfg()
    rho_ref, p_ref = 1.0, cfg.getfloat('constants', 'p0')
    hs = gamma/(gamma - 1)*p_ref/rho_ref
    be.ref_state = (rho_ref, p_ref)
    s.commit()
    uref = np.zeros(5)
    uref[0], uref[-1] = rho_ref, p_ref/(gamma - 1)
    q = u - uref[None, :, None]
    q[:, -1] -= hs*q[:, 0]
    s.ele_banks[0][0].set(q.astype(np.float32))
    s.rhs(0.0, 0, 1)
    (r,) = s.ele_scal_upts(1)

    d = disc_for_mesh(mesh, 3, ns=True)
    c = cfg.items_as('constants', float) | cfg.items_as('solver-interfaces',
                                                       float)
    ref = d.rhs_ns(u, c)
    ref[:, -1] -= hs*ref[:, 0]
    assert np.abs(r - ref).max() <= 1e-4*np.abs(ref).max()


def test_fp32_euler_rhs(built):
    from pyfr_gb300.backend import B200Backend
    from pyfr_gb300.cases import euler_vortex
    from pyfr_gb300.solvers.system import EulerSystem
    cfg, mesh = euler_vortex(n=12, order=3, precision='single')
    be = B200Backend(cfg)
    s = EulerSystem(be, mesh, None, 2, cfg)
    s.commit()
    s.rhs(0.0, 0, 1)
    (u,), (r,) = s.ele_scal_upts(0), s.ele_scal_upts(1)

    d = disc_for_mesh(mesh, 3)
    ref = d.rhs_euler(u.astype(np.float64), cfg.items_as('constants', float))
    assert np.abs(r - ref).max() <= 1e-4*np.abs(ref).max()


@pytest.mark.parametrize('case', ['vortex', 'wave'])
def test_fp32_euler_rhs_reference_shift(built, case):
    """The reference-state transform with a mean flow (Euler: the vortex's
    free stream and the mixed mesh's density wave, both moving): the FP32
    input is q = T(u - u_ref) with u_ref = (rho_ref, rho_ref V, E_ref) and
    the energy replaced by dE - h_t*drho, h_t = (E_ref + p_ref)/rho_ref;
    the kernels return T times the right-hand side with every flux formed
    from the perturbation.  Its error against the FP64 oracle must be
    several times smaller than the unshifted FP32 right-hand side's (whose
    fluxes carry the mean flow; measured 19 times on the mixed mesh, 3.7
    times on the vortex, whose own velocity is of the free stream's size), and
    within 2e-6 of the RHS scale on the vortex, 3e-5 on the mixed mesh,
    whose small tetrahedra amplify the flux rounding (1.4e-5 measured)."""
    from pyfr_gb300.backend import B200Backend
    from pyfr_gb300.cases import euler_mixed, euler_vortex
    from pyfr_gb300.solvers.system import EulerSystem
    from oracle.fr_oracle import MixedDiscretisation
    from pyfr_gb300.shapes import get_shape
    from tests.oracle_util import basis_of, ops_from_shape

    def mk():
        if case == 'vortex':
            return euler_vortex(n=12, order=3, precision='single')
        return euler_mixed(n=4, kinds='hex-pyr-tet', precision='single')

    cfg, mesh = mk()
    gamma = cfg.getfloat('constants', 'gamma')
    lhs, rhs = mesh.con
    from tests.test_oracle import MIXED_FPTS, MIXED_UPTS
    parts = {}
    for et, verts in mesh.spts.items():
        sh = get_shape(et, 3, 'gauss-legendre', 'gauss-legendre') \
            if et == 'quad' else get_shape(et, 3, MIXED_UPTS[et], MIXED_FPTS)
        parts[et] = dict(ops=ops_from_shape(sh), basis=basis_of(sh),
                         verts=verts)
    d = MixedDiscretisation(parts, zip(lhs.etypes, lhs.eidxs, lhs.fidxs),
                            zip(rhs.etypes, rhs.eidxs, rhs.fidxs),
                            periods=mesh.periods)
    c = cfg.items_as('constants', float)

    out = {}
    for shift in (False, True):
        be = B200Backend(cfg)
        s = EulerSystem(be, mesh, None, 2, cfg)
        us = {et: e.set_ics_from_cfg() for et, e in s.ele_map.items()}
        nd = mesh.ndims
        rho = np.concatenate([u[:, 0].ravel() for u in us.values()])
        mom = np.array([np.concatenate([u[:, 1 + i].ravel()
                                        for u in us.values()]).mean()
                        for i in range(nd)])
        rho_ref, p_ref = float(rho.mean()), 1.0/gamma if case == 'vortex' \
            else 1.0
        vref = mom/rho_ref
        e_ref = p_ref/(gamma - 1) + 0.5*rho_ref*float(vref @ vref)
        ht = (e_ref + p_ref)/rho_ref
        uref = np.concatenate([[rho_ref], mom, [e_ref]])
        if shift:
            be.ref_state = (rho_ref, p_ref, tuple(vref))
        s.commit()
        for j, (et, u) in enumerate(us.items()):
            q = u.copy()
            if shift:
                q = u - uref[None, :, None]
                q[:, -1] -= ht*q[:, 0]
            s.ele_banks[j][0].set(q.astype(np.float32))
        s.rhs(0.0, 0, 1)
        ref = d.rhs_euler(us, c)
        errs = []
        for (et, r), rr in zip(zip(s.ele_types, s.ele_scal_upts(1)),
                               [ref[et] for et in s.ele_types]):
            rr = rr.copy()
            if shift:
                rr[:, -1] -= ht*rr[:, 0]
            errs.append(np.abs(r - rr).max()/np.abs(rr).max())
        out[shift] = max(errs)
    assert out[True] <= (2e-6 if case == 'vortex' else 3e-5), out
    assert out[True] <= out[False]/(3 if case == 'vortex' else 5), out


@pytest.mark.parametrize('mulprec', ['native', 'bf16x3', 'bf16x3-unfused'])
@pytest.mark.parametrize('case', ['vortex', 'tgv'])
def test_mixed_rk45_l2_error(built, case, mulprec):
    from pyfr_gb300.backend import B200Backend
    from pyfr_gb300.cases import euler_vortex, ns_tgv
    from pyfr_gb300.integrators import MixedRKIntegrator
    from pyfr_gb300.solvers.system import EulerSystem, NavierStokesSystem

    if case == 'vortex':
        cfg, mesh = euler_vortex(n=10, order=3, dt=2e-3, precision='single')
        scls, nsteps, ns = EulerSystem, 20, False
    else:
        cfg, mesh = ns_tgv(n=5, order=3, dt=5e-4, precision='single')
        scls, nsteps, ns = NavierStokesSystem, 10, True
    cfg.set('backend-b200', 'mul-precision', mulprec.split('-')[0])
    if mulprec.endswith('unfused'):
        cfg.set('backend-b200', 'fuse-operators', 'false')

    be = B200Backend(cfg)
    intg = MixedRKIntegrator(be, scls, mesh, cfg)
    (u,) = intg.soln
    assert u.dtype == np.float64
    intg.run_steps(nsteps)
    (ug,) = intg.soln

    d = disc_for_mesh(mesh, 3, ns=ns)
    c = cfg.items_as('constants', float) | cfg.items_as('solver-interfaces',
                                                       float)
    rhs = (lambda x: d.rhs_ns(x, c)) if ns else (lambda x: d.rhs_euler(x, c))
    for _ in range(nsteps):
        u = rk45_step(rhs, u, intg.dt)

    assert _l2rel(ug, u) <= L2_TOL


@pytest.mark.parametrize('mul', ['native', 'bf16x3-4'])
def test_kinetic_energy_history(built, mul):
    """Kinetic-energy history of the chosen form against the FP64 plain
    form.  The history is the normalised Taylor-Green kinetic energy
    E_k = int rho |u|^2 / (2 rho0 V) (about 0.125 here); the chosen form
    must stay within 1e-8 of the FP64 value at every logged step.  Operator
    contractions in FP32 (native) or split-BF16 with four products."""
    from pyfr_gb300.backend import B200Backend
    from pyfr_gb300.cases import ns_tgv
    from pyfr_gb300.integrators import MixedRKIntegrator, RKVdH2Integrator
    from pyfr_gb300.plugins import FieldIntegrals
    from pyfr_gb300.solvers.system import NavierStokesSystem

    hist = {}
    for form, prec, icls in [('plain', 'double', RKVdH2Integrator),
                             ('chosen', 'single', MixedRKIntegrator)]:
        cfg, mesh = ns_tgv(n=6, order=3, dt=5e-4, precision=prec)
        if form == 'chosen' and mul != 'native':
            cfg.set('backend-b200', 'mul-precision', 'bf16x3')
            cfg.set('backend-b200', 'split-products', '4')
        intg = icls(B200Backend(cfg), NavierStokesSystem, mesh, cfg)
        fi = FieldIntegrals(intg)
        h = []
        for _ in range(10):
            intg.run_steps(2)
            r = fi()
            h.append(0.5*r['E']/r['vol'])
        hist[form] = np.array(h)

    assert np.abs(hist['chosen'] - hist['plain']).max() <= 1e-8


def test_autotuned_plan_same_result(built, golden, tmp_path, monkeypatch):
    """The autotuner's pipeline plan (ring depth, epilogue tiles) changes
    the schedule, not the arithmetic: results equal the default plan's bit
    for bit, and the plan is cached."""
    import ctypes as C
    import json
    from pyfr_gb300.backend import B200Backend
    from pyfr_gb300.backend import mul as mulmod
    from pyfr_gb300.inifile import Inifile
    monkeypatch.setenv('PYFR_GB300_CACHE', str(tmp_path))
    monkeypatch.setattr(mulmod, '_PLANS', None)
    a = golden['operators']['hex_p3_gauss-legendre/M460']
    rng = np.random.default_rng(9)
    b = rng.normal(size=(a.shape[1], 5, 900))
    out = {}
    for tune in ('true', 'false'):
        cfg = Inifile()
        cfg.set('backend', 'precision', 'single')
        cfg.set('backend-b200', 'mul-precision', 'bf16x3')
        cfg.set('backend-b200', 'autotune', tune)
        be = B200Backend(cfg)
        A = be.const_matrix(a)
        B = be.matrix(b.shape, b, tags={'align'})
        Cm = be.matrix((a.shape[0], 5, 900), tags={'align'})
        be.commit()
        k = be.kernel('mul', A, B, out=Cm)
        be.run_kernels([k], wait=True)
        out[tune] = Cm.get()
        ns, nt = C.c_int(), C.c_int()
        h = be._providers[2]._handles[(A.mid,)][0] if hasattr(
            be, '_providers') else None
        if h is not None:
            be.lib.mul_tc_plan(h, C.byref(ns), C.byref(nt))
            assert 4 <= ns.value <= 10
            assert nt.value in (1, 2)
    assert np.array_equal(out['true'], out['false'])
    plans = json.loads((tmp_path / 'mul-plans.json').read_text())
    assert any('|192|64|0|' in k for k in plans)


def test_chosen_form_order4(built):
    """The fused chosen-form graph at p = 4 (operators in pieces) against
    FP64 on the TGV."""
    from pyfr_gb300.backend import B200Backend
    from pyfr_gb300.cases import ns_tgv
    from pyfr_gb300.integrators import MixedRKIntegrator, RKVdH2Integrator
    from pyfr_gb300.solvers.system import NavierStokesSystem
    cfg, mesh = ns_tgv(n=4, order=4, dt=2e-4)
    plain = RKVdH2Integrator(B200Backend(cfg), NavierStokesSystem, mesh, cfg)
    cfg, mesh = ns_tgv(n=4, order=4, dt=2e-4, precision='single')
    cfg.set('backend-b200', 'mul-precision', 'bf16x3')
    cfg.set('backend-b200', 'split-products', '5')
    chosen = MixedRKIntegrator(B200Backend(cfg), NavierStokesSystem, mesh,
                               cfg)
    plain.run_steps(10)
    chosen.run_steps(10)
    (a,), (b,) = chosen.soln, plain.soln
    assert np.linalg.norm(a - b)/np.linalg.norm(b) <= 1e-6


@pytest.mark.parametrize('mulprec', ['bf16x3', 'bf16x3-unfused'])
def test_chosen_form_ns_antialiasing(built, mulprec):
    """The chosen form with Navier-Stokes flux anti-aliasing (the fused
    gradient apply, the batched M7 interpolation of the gradient, the
    unfused flux at the quadrature points on reference-state-shifted
    inputs, the fused M9 divergence): ten steps of the 5^3 Taylor-Green box
    against the FP64 plain form with anti-aliasing, within the chosen
    form's L2 bound."""
    from pyfr_gb300.backend import B200Backend
    from pyfr_gb300.cases import ns_tgv
    from pyfr_gb300.integrators import MixedRKIntegrator, RKVdH2Integrator
    from pyfr_gb300.solvers.system import NavierStokesSystem

    cfg, mesh = ns_tgv(n=5, order=3, dt=5e-4)
    cfg.set('solver', 'anti-alias', 'flux')
    plain = RKVdH2Integrator(B200Backend(cfg), NavierStokesSystem, mesh, cfg)
    cfg, mesh = ns_tgv(n=5, order=3, dt=5e-4, precision='single')
    cfg.set('solver', 'anti-alias', 'flux')
    cfg.set('backend-b200', 'mul-precision', 'bf16x3')
    cfg.set('backend-b200', 'split-products', '5')
    if mulprec.endswith('unfused'):
        cfg.set('backend-b200', 'fuse-operators', 'false')
    chosen = MixedRKIntegrator(B200Backend(cfg), NavierStokesSystem, mesh,
                               cfg)
    assert chosen.uref is not None
    plain.run_steps(10)
    chosen.run_steps(10)
    (a,), (b,) = chosen.soln, plain.soln
    assert _l2rel(a, b) <= L2_TOL


@pytest.mark.parametrize('case', ['vortex', 'tgv'])
@pytest.mark.parametrize('graphs', [True, False])
def test_stage_in_divergence_epilogue(built, case, graphs):
    """The RK stage done in the epilogue of the divergence apply (the
    right-hand side never stored) gives the solution of the separate stage
    kernel bit for bit, and the stage kernel is gone from the step."""
    from pyfr_gb300.backend import B200Backend
    from pyfr_gb300.cases import euler_vortex, ns_tgv
    from pyfr_gb300.integrators import MixedRKIntegrator
    from pyfr_gb300.solvers.system import EulerSystem, NavierStokesSystem

    sols = {}
    for fuse in ('true', 'false'):
        if case == 'vortex':
            cfg, mesh = euler_vortex(n=10, order=3, dt=2e-3,
                                     precision='single')
            scls = EulerSystem
        else:
            cfg, mesh = ns_tgv(n=5, order=3, dt=5e-4, precision='single')
            scls = NavierStokesSystem
        cfg.set('backend-b200', 'mul-precision', 'bf16x3')
        cfg.set('backend-b200', 'split-products', '5')
        cfg.set('backend-b200', 'cuda-graphs', str(graphs).lower())
        cfg.set('backend-b200', 'fuse-stage', fuse)
        intg = MixedRKIntegrator(B200Backend(cfg), scls, mesh, cfg)
        kl, _ = intg.step_kernels(intg.idxcurr, intg.dt)
        names = [k.name for k in kl]
        fused = [k for k in kl if k.meta.get('rk_stage')]
        if fuse == 'true':
            assert 'rkmixed' not in names
            assert len(fused) == intg.nstages
            assert fused[-1].meta['rk_stage'] == 2
        else:
            assert names.count('rkmixed') == intg.nstages and not fused
        intg.run_steps(6)
        (sols[fuse],) = intg.soln
    assert np.array_equal(sols['true'], sols['false'])


def _ns_rhs_single(mesh, cfg, facegrad, mul='native', shift=False):
    from pyfr_gb300.backend import B200Backend
    from pyfr_gb300.solvers.system import NavierStokesSystem
    cfg.set('backend-b200', 'face-gradients', facegrad)
    cfg.set('backend-b200', 'mul-precision', mul)
    if mul == 'bf16x3':
        cfg.set('backend-b200', 'split-products', 5)
    be = B200Backend(cfg)
    s = NavierStokesSystem(be, mesh, None, 2, cfg)
    if shift:
        # The TGV on its reference-state transform, as the chosen form runs
        gamma = cfg.getfloat('constants', 'gamma')
        rho_ref, p_ref = 1.0, cfg.getfloat('constants', 'p0')
        hs = gamma/(gamma - 1)*p_ref/rho_ref
        be.ref_state = (rho_ref, p_ref)
        (eles,) = s.ele_map.values()
        q = eles.set_ics_from_cfg() - \
            np.array([rho_ref, 0, 0, 0, p_ref/(gamma - 1)])[None, :, None]
        q[:, -1] -= hs*q[:, 0]
    s.commit()
    if shift:
        s.ele_banks[0][0].set(q.astype(np.float32))
    s.rhs(0.0, 0, 1)
    wb = {e.grad_writeback for e in s.ele_map.values()}
    return [r.astype(np.float64) for r in s.ele_scal_upts(1)], wb


@pytest.mark.parametrize('mul', ['native', 'bf16x3'])
@pytest.mark.parametrize('mesh', ['tgv', 'hex-pyr-tet', 'distorted'])
def test_face_gradients_in_reference_space(built, mul, mesh):
    """Single precision on affine elements: the flux kernel leaves the
    corrected gradient in reference space and the interface kernel
    transforms the face gradients with the elements' metric terms (one
    column per element over every type).  The right-hand side equals the
    one with the transform at the points (the reference's order) to FP32
    rounding: 1e-5 of its scale in FP32 arithmetic; the split-BF16 applies
    (the chosen form's five products) see different inputs in the two
    orders, so there their own error (2^-17 of the data, amplified by the
    operators) bounds the difference: 1e-4.  On the mixed mesh the lift of
    its small tetrahedra (1/|J| near 50) amplifies a rounding of the face
    gradients far more, against a right-hand side of 0.1: 1.0e-5 of it
    measured in FP32 (bound 1e-4) and 128 times that with the BF16 split
    data's 2^-17 (1.3e-3 measured, bound 3e-3).  A mesh with elements that
    are not affine keeps the reference's order."""
    from pyfr_gb300.cases import euler_mixed, ns_tgv
    from pyfr_gb300.mesh import mixed_box
    if mesh == 'tgv':
        mk = lambda: ns_tgv(n=4, order=3, precision='single')
    elif mesh == 'hex-pyr-tet':
        def mk():
            cfg, _ = euler_mixed(n=2, kinds='hex-pri', precision='single')
            for k, v in (('mu', 0.02), ('Pr', 0.72)):
                cfg.set('constants', k, v)
            cfg.set('solver-interfaces', 'ldg-beta', 0.5)
            cfg.set('solver-interfaces', 'ldg-tau', 0.1)
            cfg.set('soln-ics', 'u', '0.4 + 0.1*sin(y)')
            cfg.set('soln-ics', 'v', '-0.2 + 0.1*cos(z)')
            cfg.set('soln-ics', 'w', '0.1*sin(x)')
            return cfg, mixed_box(4, -np.pi, np.pi, 'hex-pyr-tet')
    else:
        def mk():
            cfg, m = ns_tgv(n=4, order=3, precision='single')
            sp = m.spts['hex']
            rng = np.random.default_rng(3)
            # Move every lattice vertex (periodic images together)
            h = 2*np.pi/4
            idx = np.rint((sp + np.pi)/h).astype(int) % 4
            jit = rng.uniform(-0.1*h, 0.1*h, size=(4, 4, 4, 3))
            sp += jit[idx[..., 0], idx[..., 1], idx[..., 2]]
            return cfg, m
    bf = mul == 'bf16x3'
    out = {}
    for fg in ('auto', 'physical'):
        cfg, m = mk()
        r, wb = _ns_rhs_single(m, cfg, fg, mul, shift=bf and mesh != 'hex-pyr-tet')
        out[fg] = r
        if fg == 'auto':
            assert wb == ({True} if mesh == 'distorted' else {False})
    tol = {(False, False): 1e-5, (True, False): 1e-4, (False, True): 1e-4,
           (True, True): 3e-3}[bf, mesh == 'hex-pyr-tet']
    for a, b in zip(out['auto'], out['physical']):
        assert np.abs(a - b).max() <= tol*np.abs(b).max()
