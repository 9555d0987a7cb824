"""Entropy filter: bounds-preserving shock capturing of the Euler and
Navier-Stokes systems (``[solver] shock-capturing = entropy-filter``).

The structure follows ``pyfr/solvers/baseadvec/entfilter.py:5-213``: each
element type holds one minimum-entropy value per face and element and a
filter strength per element; every right-hand side first filters its input
solution in place (which also stores each element's new minimum entropy),
after which the interfaces take the smaller value of their two faces and
boundaries the smaller of theirs and their ghost state's.  Before the first
step the minima are formed without filtering, and every step ends with a
filter of the new solution.

The filter acts on the orthonormal modes grouped by the largest entry of
their degree tuples: Legendre products on quadrilaterals and hexahedra,
the collapsed-coordinate bases on triangles, tetrahedra and prisms (the
reference's modes, ``pyfr/polys.py``).
"""

import ctypes as C

import numpy as np

from pyfr_gb300.backend.lib import EF
from pyfr_gb300.backend.types import Kernel
from pyfr_gb300.polys import modal_basis


class EntropyFilter:
    def __init__(self, system, cfg):
        be = self._be = system.backend
        self.system = system
        sect = 'solver-entropy-filter'
        form = cfg.get(sect, 'formulation', 'nonlinear')
        if form not in ('nonlinear', 'linearised'):
            raise ValueError('Invalid entropy filter formulation')
        self.linearise = form == 'linearised'
        self.opts = dict(
            d_min=cfg.getfloat(sect, 'd-min', 1e-6),
            p_min=cfg.getfloat(sect, 'p-min', 1e-6),
            e_tol=cfg.getfloat(sect, 'e-tol', 1e-6),
            f_tol=cfg.getfloat(sect, 'f-tol', 1e-4),
            niters=int(cfg.getfloat(sect, 'niters', 2)))
        gamma = cfg.getfloat('constants', 'gamma')

        self.entmin, self.ef_filter, self._params = {}, {}, {}
        for et, e in system.ele_map.items():
            b = e.basis
            nfaces = len(b.faces)
            init = np.full((nfaces, e.neles), -be.fpdtype_max)
            self.entmin[et] = be.matrix((nfaces, e.neles), init,
                                        extent=system.nonce + 'entmin_int',
                                        tags={'align'})
            self.ef_filter[et] = be.matrix((1, e.neles), tags={'align'})

            ub, modes, _ = modal_basis(b)
            vdm = ub.vdm                                   # (nmodes, nupts)
            invvdm = np.linalg.inv(vdm)                    # (nupts, nmodes)
            fin = bool(np.all(np.count_nonzero(b.m0, axis=1) == 1))
            vdm_ef = vdm.T if fin else \
                np.vstack([vdm.T, ub.ortho_basis_at(b.fpts).T])
            degs = np.array([max(m) for m in modes], dtype=np.int32)

            # Jacobian-weighted element mean (pyfr/solvers/base/elements.py:
            # 331-335)
            wts = invvdm[:, 0, None]/e.rcpdjac_at_np('upts')
            wts /= np.sum(wts, axis=0)

            p = EF(ndims=e.ndims, nupts=e.nupts, nfpts=e.nfpts,
                   nefpts=e.nupts + (0 if fin else e.nfpts), nfaces=nfaces,
                   order=b.order, fpts_in_upts=int(fin),
                   linearise=int(self.linearise), niters=self.opts['niters'],
                   gamma=gamma, d_min=self.opts['d_min'],
                   p_min=self.opts['p_min'], e_tol=self.opts['e_tol'],
                   f_tol=self.opts['f_tol'])
            dg = be.const_matrix(degs[None, :], dtype=np.int32)
            self._params[et] = dict(
                p=p, vdm=be.const_matrix(vdm_ef), invvdm=be.const_matrix(invvdm.T),
                m0=None if fin else be.const_matrix(b.m0),
                wts=be.const_matrix(wts, tags={'align'}), degs=dg)
        be.commit()

    # ---- kernels -------------------------------------------------------------

    def _sfx(self):
        return 'f64' if self._be.fpdtype == np.float64 else 'f32'

    def filter_kernel(self, et, u):
        be, q = self._be, self._params[et]
        fn = getattr(be.lib, f'entropyfilter_{self._sfx()}')
        e = self.system.ele_map[et]
        ent, eff = self.entmin[et], self.ef_filter[et]
        m0, ldm = (q['m0'].data, q['m0'].leaddim) if q['m0'] is not None \
            else (None, 0)
        args = (C.byref(q['p']), e.neles, u.data, u.leaddim, ent.data,
                ent.leaddim, eff.data, q['vdm'].data, q['vdm'].leaddim,
                q['invvdm'].data, q['invvdm'].leaddim, m0, ldm,
                q['wts'].data, q['wts'].leaddim, q['degs'].data)

        def run(stream):
            fn(*args, stream)

        return Kernel(run, mats=[u, ent, eff, q['vdm'], q['invvdm'],
                                 q['wts'], q['degs']] +
                      ([q['m0']] if q['m0'] is not None else []),
                      misc=[q['p']], name='entropyfilter')

    def local_kernel(self, et, u):
        be, q = self._be, self._params[et]
        fn = getattr(be.lib, f'entropylocal_{self._sfx()}')
        e = self.system.ele_map[et]
        ent = self.entmin[et]
        m0, ldm = (q['m0'].data, q['m0'].leaddim) if q['m0'] is not None \
            else (None, 0)
        args = (C.byref(q['p']), e.neles, u.data, u.leaddim, ent.data,
                ent.leaddim, m0, ldm)

        def run(stream):
            fn(*args, stream)

        return Kernel(run, mats=[u, ent], misc=[q['p']], name='entropylocal')

    def face_views(self):
        """(left, right) views of the face minima of each interior
        interface, one value per face (pyfr/solvers/baseadvec/entfilter.py:
        117-136)."""
        be, out = self._be, []
        for i in self.system._int_inters:
            views = []
            for side in (i.lhs, i.rhs):
                mm = np.array([self.entmin[t].mid for t in side.etypes.tolist()])
                views.append(be.view(mm, side.fidxs, side.eidxs, vshape=()))
            out.append(views)
        return out

    def bc_face_views(self, bc):
        """View mapping every flux point of a boundary (in the boundary's
        point order) to its face's minimum."""
        rows, cols, mats, order = [], [], [], []
        for et, fidx, eidxs, idx in bc.lhs.foreach():
            nfp = self.system.ele_map[et].nfacefpts[fidx]
            mats.append(np.full(len(eidxs)*nfp, self.entmin[et].mid))
            rows.append(np.full(len(eidxs)*nfp, fidx))
            cols.append(np.repeat(eidxs, nfp))
            order.append(np.repeat(idx, nfp))
        ro = np.argsort(np.concatenate(order), kind='stable')[bc._perm]
        return self._be.view(np.concatenate(mats)[ro],
                             np.concatenate(rows)[ro],
                             np.concatenate(cols)[ro], vshape=())

    def intcent_kernel(self, lhs, rhs):
        be = self._be
        fn = getattr(be.lib, f'intcent_{self._sfx()}')
        n = lhs.n
        args = (n, lhs.basedata, lhs.mapping.data, rhs.basedata,
                rhs.mapping.data, int(be.ixdtype == np.int64))

        def run(stream):
            fn(*args, stream)

        return Kernel(run, views=[lhs, rhs], name='intcent')

    def bccent_kernel(self, bc, entview):
        """Boundary faces take the smaller of their minimum and the entropy
        of the ghost state (pyfr/solvers/euler/kernels/bccent.mako)."""
        be = self._be
        fn = getattr(be.lib, f'bccent_{self._sfx()}')
        ul = bc.scal_lhs
        nl = bc._pnorm_lhs
        gamma = self.system.cfg.getfloat('constants', 'gamma')
        args = (bc.ndims, ul.n, gamma, C.byref(bc.bc), ul.basedata,
                ul.mapping.data, entview.basedata, entview.mapping.data,
                int(be.ixdtype == np.int64), nl.data, nl.leaddim)

        def run(stream):
            fn(*args, stream)

        return Kernel(run, mats=[nl], views=[ul, entview], misc=[bc.bc],
                      name='bccent')

    # ---- system hooks --------------------------------------------------------

    def add_kernels(self, kernels, ktags):
        """Add the filter's kernels to the system's kernel table: per bank
        'eles/entropy_filter' and 'eles/local_entropy', and
        'iint/comm_entropy', 'bcint/comm_entropy'."""
        sysm = self.system
        for et, e in sysm.ele_map.items():
            tag = f'eles/{id(e)}'
            for i in range(sysm.nrhs):
                u = e.scal_upts[i]
                for name, k in (('eles/entropy_filter',
                                 self.filter_kernel(et, u)),
                                ('eles/local_entropy',
                                 self.local_kernel(et, u))):
                    kernels[name, i, None].append(k)
                    ktags[k] = tag
        for i, (l, r) in zip(sysm._int_inters, self.face_views()):
            k = self.intcent_kernel(l, r)
            kernels['iint/comm_entropy', None, None].append(k)
            ktags[k] = f'iint/{id(i)}'
        for b in sysm._bc_inters:
            k = self.bccent_kernel(b, self.bc_face_views(b))
            kernels['bcint/comm_entropy', None, None].append(k)
            ktags[k] = f'bcint/{id(b)}'
