"""Partitions of a mesh and their shared faces (host side, no GPU).

Every interface of the whole mesh is either interior to one part or
shared by two parts that list its faces in the same order
(pyfr/solvers/base/system.py:256-263), and across two CPU ranks (gloo)
the flux points each part packs at its shared faces, exchanged with
``pyfr_gb300.exchange.TorchExchanger``, coincide with the peer's points
(modulo the periods)."""
import os

import numpy as np
import pytest

from pyfr_gb300.mesh import box, periodic_box
from pyfr_gb300.partition import gather_field, partition


def _meshes():
    return [periodic_box('quad', 6, -1.0, 1.0),
            periodic_box('hex', 4, 0.0, 2.0),
            box('hex', (3, 3, 4), 0.0, 1.0, (True, True, False))]


@pytest.mark.parametrize('mi', range(3))
@pytest.mark.parametrize('nparts', [2, 3])
def test_every_interface_once(mi, nparts):
    mesh = _meshes()[mi]
    parts = partition(mesh, nparts, axis=mesh.ndims - 1)
    ne = {et: s.shape[1] for et, s in mesh.spts.items()}
    assert sum(len(p.gidx[et]) for p in parts for et in p.gidx) == \
        sum(ne.values())

    # Interior faces of the parts and shared faces, as global faces
    seen = []
    for p in parts:
        for side in p.con:
            for t, e, f in zip(side.etypes, side.eidxs, side.fidxs):
                seen.append((str(t), int(p.gidx[t][e]), int(f)))
        for q, side in p.con_p.items():
            assert len(side) == len(parts[q].con_p[p.rank])
            for t, e, f in zip(side.etypes, side.eidxs, side.fidxs):
                seen.append((str(t), int(p.gidx[t][e]), int(f)))
    want = [(str(t), int(e), int(f)) for side in mesh.con
            for t, e, f in zip(side.etypes, side.eidxs, side.fidxs)]
    assert sorted(seen) == sorted(want)

    # Boundary faces are split, not lost
    for name, side in mesh.bcon.items():
        assert sum(len(p.bcon.get(name, [])) for p in parts) == len(side)

    # Round trip of an element field
    f = {et: np.random.default_rng(0).normal(size=(2, n))
         for et, n in ne.items()}
    local = [{et: f[et][:, p.gidx[et]] for et in p.gidx} for p in parts]
    g = gather_field(parts, local, ne)
    for et in f:
        np.testing.assert_array_equal(g[et], f[et])


def _shared_points(mesh, part, cfg):
    """The flux-point coordinates of each shared face set in the order a
    part packs them (the shared face order, each face's points sorted)."""
    from pyfr_gb300.solvers.elements import EulerElements
    from pyfr_gb300.solvers.inters import inter_arrays
    elemap = {et: EulerElements(et, part.spts[et], cfg) for et in part.spts}
    return {q: inter_arrays(side, 'get_ploc_for_inters', elemap)[0]
            for q, side in part.con_p.items()}


def _rank_main(rank, world, port, q):
    import torch.distributed as dist
    from pyfr_gb300.cases import euler_vortex
    from pyfr_gb300.exchange import TorchExchanger
    os.environ.update(MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port))
    dist.init_process_group('gloo', rank=rank, world_size=world)
    try:
        cfg, mesh = euler_vortex(n=6, order=3)
        parts = partition(mesh, world, axis=0)
        pts = _shared_points(mesh, parts[rank], cfg)
        ex = TorchExchanger()
        recv = {p: np.empty_like(a) for p, a in pts.items()}
        ex.post([(p, 7, np.ascontiguousarray(a), recv[p])
                 for p, a in sorted(pts.items())])
        ex.complete()
        per = np.asarray(mesh.periods)
        err = 0.0
        for p, a in pts.items():
            d = recv[p] - a
            d -= per*np.round(d/per)
            err = max(err, np.abs(d).max())
        q.put((rank, err, sum(len(a) for a in pts.values())))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize('world', [2, 3])
def test_exchange_pairs_points_across_ranks(world):
    import socket
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        port = s.getsockname()[1]
    ctx = mp.get_context('spawn')
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q))
             for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=300) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, err, npts in res:
        assert npts > 0
        assert err < 1e-12, (rank, err)


def _controller_rank(rank, world, port, q):
    """The step-size controllers' reductions across parts: each rank holds
    its part's error sum, DoF count and largest wave speed; the
    integrator's combination (sqrt of the summed sums over the summed DoF,
    the largest wave speed) goes through TorchExchanger.allreduce."""
    import math
    from types import SimpleNamespace
    import torch.distributed as dist
    from pyfr_gb300.exchange import TorchExchanger
    from pyfr_gb300.integrators import RKVdH2Integrator
    os.environ.update(MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port))
    dist.init_process_group('gloo', rank=rank, world_size=world)
    try:
        intg = SimpleNamespace(
            system=SimpleNamespace(_mpi_inters=[object()],
                                   exchanger=TorchExchanger()),
            gndofs=100*(rank + 1))
        intg._allreduce = lambda v, op='sum': \
            RKVdH2Integrator._allreduce(intg, v, op)
        err = RKVdH2Integrator._global_error(intg, 2.0*(rank + 1)**2)
        wmax = intg._allreduce([3.0 + rank], 'max')[0]
        q.put((rank, err, wmax))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize('world', [2, 3])
def test_controller_reductions_across_ranks(world):
    import math
    import socket
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        port = s.getsockname()[1]
    ctx = mp.get_context('spawn')
    q = ctx.Queue()
    procs = [ctx.Process(target=_controller_rank, args=(r, world, port, q))
             for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=300) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    want = math.sqrt(sum(2.0*(r + 1)**2 for r in range(world)) /
                     sum(100*(r + 1) for r in range(world)))
    for rank, err, wmax in res:
        assert abs(err - want) <= 1e-15*want, (rank, err, want)
        assert wmax == 3.0 + world - 1


def test_controller_needs_an_allreduce():
    """Parts driven in one process (LocalExchanger) cannot rendezvous: a
    controller across them is refused with a clear error."""
    from types import SimpleNamespace
    from pyfr_gb300.exchange import LocalExchanger
    from pyfr_gb300.integrators import RKVdH2Integrator
    intg = SimpleNamespace(system=SimpleNamespace(
        _mpi_inters=[object()], exchanger=LocalExchanger().endpoint(0)))
    with pytest.raises(NotImplementedError, match='allreduce'):
        RKVdH2Integrator._allreduce(intg, [1.0])
