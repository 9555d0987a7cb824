"""Artificial viscosity: shock capturing of the Navier-Stokes system
(``[solver] shock-capturing = artificial-viscosity``).

The structure follows ``pyfr/solvers/baseadvecdiff/artvisc.py:24-200``:
every right-hand side zeroes a buffer of one value per mesh vertex, a
shock sensor gives each element a viscosity from the modal content of its
density and maximises it into the element's vertices, and the vertex
values are interpolated linearly to each element's flux and solution
points.  The Navier-Stokes flux, interface flux and boundary flux then add
-mu grad u to their viscous parts.

The sensor (``pyfr/solvers/baseadvecdiff/kernels/shocksensor.mako``) is the
Klockner-Warburton-Hesthaven decay fit from order 2 up and the
Persson-Peraire modal ratio at order 1, with the constants ``max-artvisc``,
``kappa`` and ``s0`` of ``[solver-artificial-viscosity]``.  It works on the
orthonormal modes grouped by degree (``modal_basis``: the reference's modes
for every element type), with the plain integrator.
"""

import ctypes as C
import math

import numpy as np

from pyfr_gb300.backend.lib import AV
from pyfr_gb300.backend.types import Kernel
from pyfr_gb300.mesh import vertex_nodes
from pyfr_gb300.polys import modal_basis
from pyfr_gb300.shapes import linear_shape_fn


def sensor_params(modes, lower, order):
    """The sensor's per-mode degree (the largest entry of the mode's
    degree tuple), the flags of the modes missing from the basis one order
    lower, and the decay-fit weights and baseline decay of degrees
    1..order (pyfr/solvers/baseadvecdiff/artvisc.py:160-196)."""
    degs = [max(m) for m in modes]
    low = set(map(tuple, lower))
    ind = [int(tuple(m) not in low) for m in modes]
    fit = list(range(1, order + 1))
    if len(fit) >= 2:
        x = np.log(np.array(fit, dtype=float) + 1)
        a = np.column_stack([np.ones(len(x)), x])
        w = np.linalg.pinv(a)[1]
        bd = np.array([1.0/(d + 1)**(2*order) for d in fit])
        bd /= bd.sum()
    else:
        w = bd = None
    return degs, ind, w, bd


class ArtificialViscosity:
    def __init__(self, system, cfg):
        be = self._be = system.backend
        self.system = system
        sect = 'solver-artificial-viscosity'
        c = cfg.items_as(sect, float)
        for k in ('max-artvisc', 'kappa', 's0'):
            if k not in c:
                raise ValueError(f'Missing option {k!r} in [{sect}]')
        self.c = c

        vnodes, nnodes = vertex_nodes(system.mesh)
        self.nnodes = nnodes
        self.vtx = be.matrix((1, nnodes), extent=system.nonce + 'av_vtx')

        self._params = {}
        for et, e in system.ele_map.items():
            b = e.basis
            e.artvisc_fpts = be.matrix((e.nfpts, e.neles), tags={'align'},
                                       extent=system.nonce + 'artvisc_fpts')
            # (at the points of the volume flux: the solution points, or
            # the quadrature points with flux anti-aliasing)
            fpts_vol = b.qpts if e.antialias else b.upts
            e.artvisc_upts = be.matrix((len(fpts_vol), e.neles),
                                       tags={'align'})

            ub, modes, lower = modal_basis(b)
            order = b.order
            degs, ind, w, bd = sensor_params(modes, lower, order)
            invvdm = np.linalg.inv(ub.vdm).T               # (nmodes, nupts)
            nv = vnodes[et].shape[0]
            p = AV(nupts=e.nupts, nvars=e.nvars,
                   svar=list(e.convars).index('rho'), nverts=nv,
                   nmodes=len(degs), ndeg=order + 1, kwh=int(w is not None),
                   kappa=c['kappa'], max_av=c['max-artvisc'],
                   se0=math.log10(c['s0']/order**4))
            if w is not None:
                for i, (wi, bi) in enumerate(zip(w, bd)):
                    p.s_weights[i], p.baseline[i] = wi, bi
            self._params[et] = dict(
                p=p, invvdm=be.const_matrix(invvdm),
                degs=be.const_matrix(np.array([degs], dtype=np.int32),
                                     dtype=np.int32),
                ind=be.const_matrix(np.array([ind], dtype=np.int32),
                                    dtype=np.int32),
                vnodes=be.const_matrix(vnodes[et].astype(np.int32),
                                       dtype=np.int32, tags={'align'}),
                opf=be.const_matrix(linear_shape_fn(et, b.fpts)),
                opu=be.const_matrix(linear_shape_fn(et, fpts_vol)))
        be.commit()

    def _sfx(self):
        return 'f64' if self._be.fpdtype == np.float64 else 'f32'

    # ---- kernels -------------------------------------------------------------

    def zero_kernel(self):
        lib, v = self._be.lib, self.vtx
        nbytes = v.nrow*v.leaddim*v.itemsize

        def run(stream):
            lib.memset(v.data, 0, nbytes, stream)

        return Kernel(run, mats=[v], name='vtx_zero')

    def sensor_kernel(self, et, u):
        q, e = self._params[et], self.system.ele_map[et]
        fn = getattr(self._be.lib, f'shocksensor_{self._sfx()}')
        args = (C.byref(q['p']), e.neles, u.data, u.leaddim, q['invvdm'].data,
                q['invvdm'].leaddim, q['degs'].data, q['ind'].data,
                q['vnodes'].data, q['vnodes'].leaddim, self.vtx.data)

        def run(stream):
            fn(*args, stream)

        return Kernel(run, mats=[u, self.vtx, q['invvdm'], q['degs'],
                                 q['ind'], q['vnodes']], misc=[q['p']],
                      name='shocksensor')

    def fill_kernel(self, et):
        q, e = self._params[et], self.system.ele_map[et]
        fn = getattr(self._be.lib, f'avfill_{self._sfx()}')
        nv = q['p'].nverts
        calls = [(nv, op.nrow, e.neles, self.vtx.data, q['vnodes'].data,
                  q['vnodes'].leaddim, op.data, op.leaddim, out.data,
                  out.leaddim)
                 for op, out in ((q['opf'], e.artvisc_fpts),
                                 (q['opu'], e.artvisc_upts))]

        def run(stream):
            for a in calls:
                fn(*a, stream)

        return Kernel(run, mats=[self.vtx, q['vnodes'], q['opf'], q['opu'],
                                 e.artvisc_fpts, e.artvisc_upts],
                      name='avfill')

    def vertex_values(self):
        """The viscosity of every vertex (the exported field of
        pyfr/solvers/baseadvecdiff/elements.py:125-131)."""
        return self.vtx.get().ravel()[:self.nnodes]

    # ---- system hooks --------------------------------------------------------

    def add_kernels(self, kernels, ktags):
        """Kernels 'vtx/vtx_zero', per bank 'eles/shocksensor', and
        'eles/avfill'."""
        sysm = self.system
        k = self.zero_kernel()
        kernels['vtx/vtx_zero', None, None].append(k)
        ktags[k] = 'vtx'
        for et, e in sysm.ele_map.items():
            tag = f'eles/{id(e)}'
            for i in range(sysm.nrhs):
                k = self.sensor_kernel(et, e.scal_upts[i])
                kernels['eles/shocksensor', i, None].append(k)
                ktags[k] = tag
            k = self.fill_kernel(et)
            kernels['eles/avfill', None, None].append(k)
            ktags[k] = tag
