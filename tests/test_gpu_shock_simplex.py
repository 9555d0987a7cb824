"""Shock capturing on triangles, tetrahedra, prisms and pyramids (the
orthonormal modal bases of pyfr/polys.py grouped by degree, as
pyfr/solvers/baseadvec/entfilter.py:93-116 and
pyfr/solvers/baseadvecdiff/artvisc.py:160-196 group them).

* The entropy filter kernel: the face minima are formed from a smooth
  state, the density is then perturbed so that elements break their
  entropy bound, and one filter pass must match the oracle's per-element
  filter (relative max-norm 1e-10 on the solution, the strengths and the
  new minima).
* The shock sensor and the viscosity fill on a Navier-Stokes system: the
  vertex values and the viscosity at the flux points against the oracle's
  (1e-12)."""
from types import SimpleNamespace

import numpy as np
import pytest

from oracle.fr_oracle import EntropyFilterOracle, artvisc_points, shock_sensor

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def built():
    import __graft_entry__ as ge
    ge.build_library()


def _relerr(a, b):
    return np.abs(a - b).max()/max(np.abs(b).max(), 1e-300)


MESHES = ['tri', 'pri-tet', 'hex-pri', 'hex-pyr-tet']


def _mesh(kinds):
    from pyfr_gb300.mesh import mixed_box, tri_box
    return tri_box(6, -1.0, 1.0) if kinds == 'tri' else \
        mixed_box(4, -1.0, 1.0, kinds)


def _cfg(ndims, extra):
    from pyfr_gb300.cases import euler_mixed
    cfg, _ = euler_mixed(n=2, kinds='hex-pri')
    cfg.set('constants', 'mu', 0.01)
    cfg.set('constants', 'Pr', 0.72)
    cfg.set('solver-interfaces', 'ldg-beta', 0.5)
    cfg.set('solver-interfaces', 'ldg-tau', 0.1)
    r2 = 'x*x + y*y' + (' + z*z' if ndims == 3 else '')
    cfg.set('soln-ics', 'rho', f'1 + 0.4*tanh(8*({r2} - 0.3))')
    cfg.set('soln-ics', 'p', f'1 + 0.3*tanh(8*({r2} - 0.3))')
    if ndims == 2:
        for k in ('w',):
            cfg._cp.remove_option('soln-ics', k)
    for (sect, k), v in extra.items():
        cfg.set(sect, k, v)
    return cfg


@pytest.mark.parametrize('kinds', MESHES)
def test_entropy_filter_simplex(built, kinds):
    from pyfr_gb300.backend import B200Backend
    from pyfr_gb300.polys import modal_basis
    from pyfr_gb300.solvers.system import EulerSystem

    mesh = _mesh(kinds)
    cfg = _cfg(mesh.ndims, {('solver', 'shock-capturing'): 'entropy-filter'})
    be = B200Backend(cfg)
    s = EulerSystem(be, mesh, None, 2, cfg)
    s.commit()
    ef = s._ef
    for k in s.preproc_kernels(0):
        k.run(be.stream)
    be.wait()
    ent0 = {et: ef.entmin[et].get() for et in s.ele_types}

    rng = np.random.default_rng(11)
    upert = {}
    for et, e, m in zip(s.ele_types, s.ele_map.values(), s.ele_scal_upts(0)):
        u = m.copy()
        hit = rng.random(u.shape[2]) < 0.3
        u[:, 0, hit] *= 1 + 0.25*rng.standard_normal(u[:, 0, hit].shape)
        u[:, 0] = np.maximum(u[:, 0], 0.3)
        upert[et] = u
        s.ele_banks[s.ele_types.index(et)][0].set(u)
    for k in s._get_kernels(0, None)['eles/entropy_filter']:
        k.run(be.stream)
    be.wait()

    nfilt = 0
    for j, (et, e) in enumerate(s.ele_map.items()):
        b = e.basis
        ub, modes, _ = modal_basis(b)
        invvdm = np.linalg.inv(ub.vdm)
        fin = bool(np.all(np.count_nonzero(b.m0, axis=1) == 1))
        vdm = ub.vdm.T if fin else \
            np.vstack([ub.vdm.T, ub.ortho_basis_at(b.fpts).T])
        wts = invvdm[:, 0, None]/e.rcpdjac_at_np('upts')
        wts /= wts.sum(axis=0)
        ops = dict(vdm=vdm, invvdm=invvdm.T, m0=None if fin else b.m0,
                   mean_wts=wts, degs=np.array([max(m) for m in modes]))
        opts = dict(d_min=1e-6, p_min=1e-6, e_tol=1e-6, f_tol=1e-4,
                    niters=2, order=b.order, linearise=False)
        disc = SimpleNamespace(facefpts=b.facefpts, neles=e.neles)
        o = EntropyFilterOracle(disc, ops, opts, 1.4)
        o.entmin = ent0[et]
        u = upert[et].copy()
        fs, emins = [], []
        for i in range(e.neles):
            ue = u[:, :, i].copy()
            f, emin = o.filter_element(ue, i)
            u[:, :, i] = ue
            fs.append(f)
            emins.append(emin)
        fs = np.array(fs)
        nfilt += int(np.sum(fs < 1))
        assert _relerr(s.ele_banks[j][0].get(), u) < 1e-10, et
        assert _relerr(ef.ef_filter[et].get()[0], fs) < 1e-10, et
        assert _relerr(ef.entmin[et].get()[0], np.array(emins)) < 1e-10, et
    assert nfilt > 0


@pytest.mark.parametrize('kinds', MESHES)
def test_shock_sensor_simplex(built, kinds):
    from pyfr_gb300.backend import B200Backend
    from pyfr_gb300.mesh import vertex_nodes
    from pyfr_gb300.polys import modal_basis
    from pyfr_gb300.shapes import linear_shape_fn
    from pyfr_gb300.solvers.artvisc import sensor_params
    from pyfr_gb300.solvers.system import NavierStokesSystem

    mesh = _mesh(kinds)
    c = {'max-artvisc': 0.01, 'kappa': 1.2, 's0': 0.01}
    extra = {('solver', 'shock-capturing'): 'artificial-viscosity'}
    extra |= {('solver-artificial-viscosity', k): v for k, v in c.items()}
    cfg = _cfg(mesh.ndims, extra)
    be = B200Backend(cfg)
    s = NavierStokesSystem(be, mesh, None, 2, cfg)
    s.commit()
    s.rhs(0.0, 0, 1)

    vn, nn = vertex_nodes(mesh)
    vtx = np.zeros(nn)
    avs, mus = {}, []
    for et, e, u in zip(s.ele_types, s.ele_map.values(), s.ele_scal_upts(0)):
        b = e.basis
        ub, modes, lower = modal_basis(b)
        degs, *_ = sensor_params(modes, lower, b.order)
        av = dict(invvdm=np.linalg.inv(ub.vdm).T, degs=degs, order=b.order,
                  c=c, vnodes=vn[et], nnodes=nn,
                  opf=linear_shape_fn(et, b.fpts),
                  opu=linear_shape_fn(et, b.upts))
        mu = shock_sensor(u, av)
        mus.append(mu)
        np.maximum.at(vtx, vn[et].ravel(),
                      np.broadcast_to(mu, vn[et].shape).ravel())
        avs[et] = av
    assert np.any(np.concatenate(mus) > 0)
    assert _relerr(s._av.vertex_values(), vtx) < 1e-12
    for et, e in s.ele_map.items():
        ve = vtx[vn[et]]
        assert _relerr(e.artvisc_fpts.get(), avs[et]['opf'] @ ve) < 1e-12
