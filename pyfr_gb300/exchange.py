"""Exchange of packed face data between partitions.

A partition packs the solution (and, for Navier-Stokes, the gradient) at
the faces it shares with each neighbour into a device buffer, copies it to
the host, and sends it; it receives the neighbour's buffer for the same
faces, in the same order, and copies it to the device, where the interface
kernels read it through a view (the reference's persistent MPI requests
between its pack and unpack kernels, pyfr/solvers/base/system.py:185-202,
pyfr/backends/base/types.py XchgMatrix/XchgView).

``post`` starts every transfer of one exchange and ``complete`` finishes
them, so that parts driven from one process can post all their sends
before any of them waits.

* ``TorchExchanger``: one process per partition over ``torch.distributed``
  (gloo for host buffers), point-to-point with one tag per field.
* ``LocalExchanger``: several partitions in one process (one GPU, or
  tests); a posted buffer waits in a mailbox until its peer completes.

``allreduce`` (``TorchExchanger``) combines the step-size controllers'
per-part sums and maxima; parts driven in one process have no blocking
rendezvous, so the controllers need one process per part.
"""


class TorchExchanger:
    def __init__(self, group=None):
        self.group = group
        self._reqs = []

    def post(self, items):
        """items: (peer rank, tag, send array, receive array) tuples of
        host arrays."""
        import torch
        import torch.distributed as dist
        for peer, tag, sbuf, rbuf in items:
            self._reqs.append(dist.isend(torch.from_numpy(sbuf), peer,
                                         group=self.group, tag=tag))
            self._reqs.append(dist.irecv(torch.from_numpy(rbuf), peer,
                                         group=self.group, tag=tag))

    def complete(self):
        for r in self._reqs:
            r.wait()
        self._reqs = []

    def allreduce(self, values, op='sum'):
        """Sum (or maximum, op='max') of ``values`` over every rank of the
        group: the step-size controllers' global error norm and wave
        speed (the reference's MPI Allreduce, pyfr/integrators/
        controllers.py:105-117 and 22-26)."""
        import numpy as np
        import torch
        import torch.distributed as dist
        t = torch.tensor(np.asarray(values, dtype=np.float64))
        dist.all_reduce(t, op={'sum': dist.ReduceOp.SUM,
                               'max': dist.ReduceOp.MAX}[op],
                        group=self.group)
        return t.numpy()


class LocalExchanger:
    """The mailboxes of the partitions of one process; ``endpoint(rank)``
    is the exchanger of partition ``rank``."""

    def __init__(self):
        self.mail = {}

    def endpoint(self, rank):
        return _LocalEndpoint(self, rank)


class _LocalEndpoint:
    def __init__(self, hub, rank):
        self.hub, self.rank = hub, rank
        self._items = []

    def post(self, items):
        for peer, tag, sbuf, rbuf in items:
            key = (self.rank, peer, tag)
            if key in self.hub.mail:
                raise RuntimeError(f'Unreceived buffer {key}')
            self.hub.mail[key] = sbuf.copy()
        self._items = list(items)

    def complete(self):
        for peer, tag, sbuf, rbuf in self._items:
            try:
                data = self.hub.mail.pop((peer, self.rank, tag))
            except KeyError:
                raise RuntimeError(f'Partition {peer} has not sent tag {tag} '
                                   f'to {self.rank}') from None
            if data.shape != rbuf.shape:
                raise ValueError('Exchange buffers differ in size')
            rbuf[...] = data
        self._items = []
