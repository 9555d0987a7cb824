"""Artificial viscosity: host logic and the oracle (CPU).

The sensor follows pyfr/solvers/baseadvecdiff/kernels/shocksensor.mako
with the parameters of pyfr/solvers/baseadvecdiff/artvisc.py:160-196."""
import numpy as np
import pytest

from oracle.fr_oracle import artvisc_points, shock_sensor
from pyfr_gb300.mesh import box, mixed_box, periodic_box, vertex_nodes
from pyfr_gb300.shapes import get_shape, linear_shape_fn
from pyfr_gb300.polys import modal_basis
from pyfr_gb300.solvers.artvisc import sensor_params
from tests.oracle_util import disc_for_mesh


def av_case(et, mesh, order, c, seed=5):
    """Sensor parameters and a density with a smooth part, a steep front
    and a noisy band: the three branches of the sensor (zero, smooth ramp,
    maximum) all occur."""
    nd = mesh.ndims
    s = get_shape(et, order, 'gauss-legendre', 'gauss-legendre')
    degs, ind, w, bd = sensor_params(*modal_basis(s)[1:], order)
    vn, nn = vertex_nodes(mesh)
    av = dict(invvdm=np.linalg.inv(s.ubasis.vdm).T, degs=degs, order=order,
              c=c, vnodes=vn[et], nnodes=nn, opf=linear_shape_fn(et, s.fpts),
              opu=linear_shape_fn(et, s.upts))
    x = np.einsum('pv,ved->pde', linear_shape_fn(et, s.upts), mesh.spts[et])
    rng = np.random.default_rng(seed)
    rho = 1 + 0.3*np.tanh((x[:, 0] - 0.55)/0.01) + \
        0.05*np.sin(2*np.pi*x[:, 1])
    noisy = x[:, 0].mean(axis=0) < 0.3
    rho[:, noisy] += 0.05*rng.standard_normal(rho[:, noisy].shape)
    u = np.zeros((s.nupts, nd + 2, x.shape[2]))
    vel = np.array([0.2, -0.1, 0.05])[:nd]
    u[:, 0] = rho
    u[:, 1:nd + 1] = rho[:, None]*vel[None, :, None]
    u[:, -1] = 1.0/0.4 + 0.5*rho*(vel @ vel)
    return av, u


def test_vertex_nodes():
    m = periodic_box('hex', (3, 2, 2), 0.0, 1.0)
    vn, nn = vertex_nodes(m)
    assert nn == 4*3*3 and vn['hex'].shape == (8, 12)
    # Each interior node of the 3x2x2 grid is shared by its 8 cells
    counts = np.bincount(vn['hex'].ravel(), minlength=nn)
    assert counts.max() == 8 and counts.sum() == 96
    m = mixed_box(2, -1.0, 1.0, 'hex-pri')
    vn, nn = vertex_nodes(m)
    assert nn == 27 and set(vn) == {'hex', 'pri'}


def test_sensor_params():
    s = get_shape('hex', 3)
    degs, ind, w, bd = sensor_params(*modal_basis(s)[1:], 3)
    assert len(degs) == 64 and max(degs) == 3 and sum(ind) == 64 - 27
    # Least-squares slope of ln(e) against ln(d + 1): w . ln(d + 1) = 1
    assert np.isclose(w @ np.log(np.arange(2, 5)), 1.0)
    assert np.isclose(w.sum(), 0.0) and np.isclose(bd.sum(), 1.0)
    assert sensor_params(*modal_basis(get_shape('quad', 1))[1:], 1)[2] is None


# Sensor constants per order: the decay fit's rate stays near 2.3-3 for a
# positive density (the baseline decay keeps it from the maximum branch),
# so kappa = 0.9 splits smooth elements (zero) from the front (the ramp);
# the modal ratio at order 1 reaches all three branches with s0 = 1e-4
AV_C = {1: {'max-artvisc': 0.01, 'kappa': 0.5, 's0': 1e-4},
        2: {'max-artvisc': 0.01, 'kappa': 0.9, 's0': 0.01},
        3: {'max-artvisc': 0.01, 'kappa': 0.9, 's0': 0.01}}


@pytest.mark.parametrize('et,n,order', [('hex', 4, 3), ('quad', 8, 2),
                                        ('quad', 8, 1)])
def test_sensor_branches(et, n, order):
    mesh = periodic_box(et, n, 0.0, 1.0)
    av, u = av_case(et, mesh, order, AV_C[order])
    mu = shock_sensor(u, av)
    assert np.all((mu >= 0) & (mu <= 0.01))
    assert np.any((mu > 0) & (mu < 0.01))
    if order == 1:
        assert np.any(mu == 0) and np.any(mu == 0.01)
    # Vertex maxima interpolate linearly: within [0, max] everywhere
    avf, avu = artvisc_points(mu, av)
    assert avf.min() >= 0 and avu.max() <= 0.01 + 1e-15


def test_zero_viscosity_is_plain_ns():
    """max-artvisc = 0 leaves the Navier-Stokes RHS unchanged."""
    et = 'quad'
    mesh = periodic_box(et, 4, 0.0, 1.0)
    av, u = av_case(et, mesh, 3, {'max-artvisc': 0.0, 'kappa': 0.9,
                                  's0': 0.01})
    d = disc_for_mesh(mesh, 3, ns=True)
    c = dict(gamma=1.4, mu=0.01, Pr=0.72, **{'ldg-beta': 0.5,
                                             'ldg-tau': 0.1})
    assert np.array_equal(d.rhs_ns(u, c), d.rhs_ns(u, c, av=av))
