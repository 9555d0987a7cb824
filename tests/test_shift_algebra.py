"""The reference-state transform's flux algebra (the shifted flux of
pyfr_gb300/csrc/physics.cuh, inviscid_flux_shift) restated in numpy and
checked against its definition: with q = T(u - u_ref), u_ref = (rho_ref,
rho_ref V, E_ref), E_ref = p_ref/(gamma - 1) + rho_ref |V|^2/2, and T the
energy row minus h_t = (E_ref + p_ref)/rho_ref times the mass row, the
perturbation forms of the fluxes equal T (F(u) - F(u_ref)) to FP64
rounding, for a fluid at rest (V = 0, the Navier-Stokes kernels' case) and
a moving one.  No GPU."""
import numpy as np
import pytest

GAMMA = 1.4


def euler_flux(u):
    """F[d, v, n] of states u[v, n]."""
    nd = u.shape[0] - 2
    rho, m, E = u[0], u[1:-1], u[-1]
    v = m/rho
    p = (GAMMA - 1)*(E - 0.5*np.einsum('dn,dn->n', m, v))
    f = np.empty((nd, nd + 2, u.shape[1]))
    f[:, 0] = m
    for j in range(nd):
        f[:, j + 1] = m[j]*v
        f[j, j + 1] += p
    f[:, -1] = (E + p)*v
    return f


def shifted_flux(q, rho_ref, p_ref, vref):
    """The perturbation forms: rho = rho_ref + q0, dm = q[1:-1],
    dE = qE + h_t q0, w = (dm - V q0)/rho, v = V + w, dp = (gamma - 1)(dE -
    (rho_ref V.w + dm.v)/2); fluxes dm, rho_ref V w + dm v + dp I and
    (qE + dp) v."""
    nd = q.shape[0] - 2
    mref = rho_ref*vref
    e_ref = p_ref/(GAMMA - 1) + 0.5*rho_ref*vref @ vref
    ht = (e_ref + p_ref)/rho_ref
    rho = rho_ref + q[0]
    dm, dE = q[1:-1], q[-1] + ht*q[0]
    w = (dm - vref[:, None]*q[0])/rho
    v = vref[:, None] + w
    dp = (GAMMA - 1)*(dE - 0.5*(np.einsum('d,dn->n', mref, w) +
                                np.einsum('dn,dn->n', dm, v)))
    f = np.empty((nd, nd + 2, q.shape[1]))
    f[:, 0] = dm
    for i in range(nd):
        for j in range(nd):
            f[i, j + 1] = mref[i]*w[j] + dm[i]*v[j] + (dp if i == j else 0)
    f[:, -1] = (q[-1] + dp)*v
    return f


@pytest.mark.parametrize('nd', [2, 3])
@pytest.mark.parametrize('moving', [False, True])
def test_shifted_flux_is_the_transformed_flux_difference(nd, moving):
    rng = np.random.default_rng(nd + 10*moving)
    n = 200
    rho_ref, p_ref = 1.1, 0.9
    vref = rng.uniform(-1, 1, nd) if moving else np.zeros(nd)
    rho = rho_ref*(1 + 0.2*rng.uniform(-1, 1, n))
    vel = vref[:, None] + 0.3*rng.normal(size=(nd, n))
    p = p_ref*(1 + 0.2*rng.uniform(-1, 1, n))
    u = np.vstack([rho, rho*vel, p/(GAMMA - 1) + 0.5*rho*(vel*vel).sum(0)])

    e_ref = p_ref/(GAMMA - 1) + 0.5*rho_ref*vref @ vref
    uref = np.concatenate([[rho_ref], rho_ref*vref, [e_ref]])
    ht = (e_ref + p_ref)/rho_ref
    q = u - uref[:, None]
    q[-1] -= ht*q[0]

    want = euler_flux(u) - euler_flux(np.repeat(uref[:, None], n, 1))
    want[:, -1] -= ht*want[:, 0]
    got = shifted_flux(q, rho_ref, p_ref, vref)
    np.testing.assert_allclose(got, want, rtol=0,
                               atol=1e-13*np.abs(euler_flux(u)).max())


def test_shifted_flux_rounds_with_the_perturbation():
    """In FP32 the perturbation forms of a moving flow carry rounding of
    the perturbation's size, the direct flux difference that of the mean
    flux: on a state 1e-3 away from the reference, the shifted FP32 flux
    is over a hundred times closer to the exact difference."""
    rng = np.random.default_rng(5)
    n, nd = 500, 3
    rho_ref, p_ref = 1.0, 1.0
    vref = np.array([1.0, 0.5, 0.25])
    rho = rho_ref*(1 + 1e-3*rng.uniform(-1, 1, n))
    vel = vref[:, None] + 1e-3*rng.normal(size=(nd, n))
    p = p_ref*(1 + 1e-3*rng.uniform(-1, 1, n))
    u = np.vstack([rho, rho*vel, p/(GAMMA - 1) + 0.5*rho*(vel*vel).sum(0)])
    e_ref = p_ref/(GAMMA - 1) + 0.5*rho_ref*vref @ vref
    uref = np.concatenate([[rho_ref], rho_ref*vref, [e_ref]])
    ht = (e_ref + p_ref)/rho_ref
    q = u - uref[:, None]
    q[-1] -= ht*q[0]

    exact = euler_flux(u) - euler_flux(np.repeat(uref[:, None], n, 1))
    exact[:, -1] -= ht*exact[:, 0]
    f32 = np.float32
    direct = (euler_flux(u.astype(f32)).astype(float) -
              euler_flux(np.repeat(uref[:, None], n, 1).astype(f32)))
    direct[:, -1] -= ht*direct[:, 0]
    shifted = shifted_flux(q.astype(f32), f32(rho_ref), f32(p_ref),
                           vref.astype(f32)).astype(float)
    e_direct = np.abs(direct - exact).max()
    e_shift = np.abs(shifted - exact).max()
    assert e_shift*100 < e_direct, (e_shift, e_direct)
