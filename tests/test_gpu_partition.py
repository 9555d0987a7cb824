"""Partitions with exchanged face data (pyfr/solvers/baseadvec/
inters.py:31-47, pyfr/solvers/baseadvecdiff/inters.py:33-60,
mpicflux.mako, mpiconu.mako) on one GPU: the parts of a mesh, driven in
lockstep from one process through ``pyfr_gb300.exchange.LocalExchanger``
(packing kernel, host transfer, interface kernels reading the received
data through a view), give the right-hand side of the whole mesh to 1e-12
relative.  Navier-Stokes uses ldg-beta = 0: with beta = +-1/2 the common
solution at a shared face is taken from the side the partitions' ranks
select (the reference's rule), not from the whole mesh's right side."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def built():
    import __graft_entry__ as ge
    ge.build_library()


def _case(name):
    from pyfr_gb300.cases import euler_vortex, ns_tgv
    from pyfr_gb300.solvers.system import EulerSystem, NavierStokesSystem
    if name == 'vortex':
        cfg, mesh = euler_vortex(n=8, order=3)
        return cfg, mesh, EulerSystem, 0
    if name == 'tgv':
        cfg, mesh = ns_tgv(n=4, order=3, beta=0.0)
        return cfg, mesh, NavierStokesSystem, 2
    from tests.bc_cases import bc_case
    cfg, mesh, _ = bc_case('ns', ('no-slp-isot-wall', 'char-riem-inv'))
    cfg.set('solver-interfaces', 'ldg-beta', 0.0)
    return cfg, mesh, NavierStokesSystem, 2


@pytest.mark.parametrize('nparts', [2, 3])
@pytest.mark.parametrize('name', ['vortex', 'tgv', 'bc-ns'])
def test_partitioned_rhs(built, name, nparts):
    from pyfr_gb300.backend import B200Backend
    from pyfr_gb300.exchange import LocalExchanger
    from pyfr_gb300.partition import gather_field, partition

    cfg, mesh, cls, axis = _case(name)
    whole = cls(B200Backend(cfg), mesh, None, 2, cfg)
    whole.commit()
    whole.rhs(0.0, 0, 1)
    want = dict(zip(whole.ele_types, whole.ele_scal_upts(1)))

    be = B200Backend(cfg)
    parts = partition(mesh, nparts, axis=axis)
    hub = LocalExchanger()
    systems = []
    for pm in parts:
        s = cls(be, pm, None, 2, cfg)
        s.exchanger = hub.endpoint(pm.rank)
        s.commit()
        assert s._mpi_inters
        systems.append(s)
    phases = [s.rhs_phases(0.0, 0, 1) for s in systems]
    assert len({len(p) for p in phases}) == 1
    for step in zip(*phases):
        for f in step:
            f()
    assert not hub.mail
    got = gather_field(parts, [dict(zip(s.ele_types, s.ele_scal_upts(1)))
                               for s in systems],
                       {et: sp.shape[1] for et, sp in mesh.spts.items()})
    for et in want:
        err = np.abs(got[et] - want[et]).max()/np.abs(want[et]).max()
        assert err < 1e-12, (et, err)


def test_partition_launches_pack_kernels(built):
    """The shared faces' data goes through the packing kernel and the
    interface kernels read the received data (the graphs hold pack and
    mpicflux kernels, the exchanges are host steps)."""
    from pyfr_gb300.backend import B200Backend
    from pyfr_gb300.partition import partition
    from pyfr_gb300.solvers.system import HostStep
    cfg, mesh, cls, _ = _case('tgv')
    (pm, _) = partition(mesh, 2, axis=2)
    s = cls(B200Backend(cfg), pm, None, 2, cfg)
    s.commit()
    gs = s.rhs_graphs(0, 1)
    hosts = [g for g in gs if isinstance(g, HostStep)]
    assert len(hosts) == 2
    names = [k.name for g in gs if not isinstance(g, HostStep)
             for k in g.klist]
    assert names.count('pack') == 2
