"""Systems: element loading, register banks, interface views, kernel
generation and the per-RHS dependency graphs.

``EulerSystem.rhs`` runs two graphs and ``NavierStokesSystem.rhs`` three,
with the kernel order, dependencies and fusion groups of
``pyfr/solvers/baseadvec/system.py:57-136`` and
``pyfr/solvers/baseadvecdiff/system.py:53-231``; the gradient-only pass
for diagnostics follows ``pyfr/solvers/baseadvecdiff/system.py:233-286``.
"""

from collections import defaultdict
from itertools import count, zip_longest
import inspect

import numpy as np

from pyfr_gb300.backend.types import Kernel, NullKernel
from pyfr_gb300.solvers.elements import EulerElements, NavierStokesElements
from pyfr_gb300.solvers.inters import (EulerBCInters, EulerIntInters,
                                       EulerMPIInters, NavierStokesBCInters,
                                       NavierStokesIntInters,
                                       NavierStokesMPIInters,
                                       field_view_arrays)


class HostStep:
    """A step between graphs that the host runs (the exchange of packed
    face data with other partitions): its kernels post and complete the
    transfers.  It runs like a graph but is never captured."""

    def __init__(self, post, complete, name):
        self.klist = [Kernel(post, name=f'{name}_post'),
                      Kernel(complete, name=f'{name}_complete')]

    def run(self, stream):
        for k in self.klist:
            k.run(stream)


class BaseSystem:
    elementscls = None
    intinterscls = None
    _nonce_seq = count()

    def __init__(self, backend, mesh, initsoln, nregs, cfg, needs_cfl=False):
        self.backend = backend
        self._needs_cfl = needs_cfl
        self.mesh = mesh
        self.cfg = cfg
        self.ndims = mesh.ndims
        self.nonce = nonce = str(next(self._nonce_seq))

        # Elements and initial conditions
        elemap = {et: self.elementscls(et, spts, cfg)
                  for et, spts in mesh.spts.items()}
        eles = list(elemap.values())
        self.nvars = eles[0].nvars

        if initsoln is not None:
            ics = [np.asarray(initsoln[et]) for et in elemap]
        else:
            ics = [e.set_ics_from_cfg() for e in eles]

        for et, e in elemap.items():
            curved = mesh.spts_curved.get(et, np.zeros(e.neles, dtype=bool))
            linoff = np.max(*np.nonzero(curved), initial=-1) + 1
            e.set_backend(backend, nonce, linoff)
            if needs_cfl:
                e.init_wavespeed()
        backend.commit()

        self.ele_map = elemap
        self.ele_types = list(elemap)
        self.ele_ndofs = [e.neles*e.nupts*e.nvars for e in eles]
        self.ele_shapes = {et: (e.nupts, e.nvars, e.neles)
                           for et, e in elemap.items()}
        self.ele_ploc_upts = [e.ploc_at_np('upts') for e in eles]

        # Register banks (all of them hold right-hand-side data)
        self.nrhs = nregs
        self.ele_banks = [[e.alloc_bank(f'bank_{id(e)}_{i}',
                                        ic if i == 0 else None)
                           for i in range(nregs)] for e, ic in zip(eles, ics)]
        backend.commit()

        lhs, rhs = mesh.con
        self._int_inters = [self.intinterscls(backend, lhs, rhs, elemap, cfg)]

        # Faces shared with other partitions (a part of
        # pyfr_gb300.partition.partition: its rank and con_p)
        self.rank = getattr(mesh, 'rank', 0)
        self._mpi_inters = [
            self.mpiinterscls(backend, side, peer, elemap, cfg, self.rank)
            for peer, side in sorted(getattr(mesh, 'con_p', {}).items())]
        # (set before the first right-hand side: pyfr_gb300.exchange)
        self.exchanger = None

        # Boundaries: one interface object per named boundary, its type from
        # [soln-bcs-<name>] (pyfr/solvers/base/system.py:183-198)
        # The step-start and stage times (device memory) that boundary
        # values given as expressions of t read
        self._tmat = backend.matrix((1, 2), dtype=np.float64)

        self._bc_inters = []
        for name, side in sorted(getattr(mesh, 'bcon', {}).items()):
            sect = f'soln-bcs-{name}'
            if not cfg.hassect(sect):
                raise ValueError(f'No [{sect}] section for boundary {name!r}')
            self._bc_inters.append(self.bcinterscls(backend, side, elemap,
                                                    sect, cfg))

    @property
    def gndofs(self):
        return sum(self.ele_ndofs)

    @property
    def _sided_inters(self):
        return self._int_inters + self._mpi_inters + self._bc_inters

    def make_field_views(self, field, vshape=()):
        """(left, right) views of a flux-point field for every interior
        interface, then (left,) for every interface with another partition
        and every boundary."""
        out = []
        for i in self._sided_inters:
            views = []
            for side in (i.lhs, i.rhs):
                if side is None:
                    continue
                m, r, c = field_view_arrays(side, field, self.ele_map)
                p = i._perm
                views.append(self.backend.view(m[p], r[p], c[p],
                                               vshape=vshape))
            out.append(tuple(views))
        return out

    def _interfaces_cover_fpts(self):
        """True when every face of every element is one side of an interior
        interface (a fully periodic mesh): the common solution can then be
        written to both sides of each interface point with no copy."""
        nside = defaultdict(int)
        for i in self._sided_inters:
            for side in (i.lhs, i.rhs):
                if side is None:
                    continue
                for et in side.etypes.tolist():
                    nside[et] += 1
        return all(nside[et] == e.neles*len(e.basis.faces)
                   for et, e in self.ele_map.items())

    def commit(self):
        covered = self._interfaces_cover_fpts()
        for e in self.ele_map.values():
            e.comm_covered = covered
        for i in self._int_inters:
            i.covers = covered
        scal = {et: e._scal_fpts for et, e in self.ele_map.items()}
        for i, v in zip(self._sided_inters,
                        self.make_field_views(scal, vshape=(self.nvars,))):
            i.scal_lhs = v[0]
            i.scal_rhs = v[1] if len(v) > 1 else None

        # Shock capturing by artificial viscosity: its fields exist before
        # the flux kernels that read them are made
        # (pyfr/solvers/baseadvecdiff/system.py:9-34)
        sc = self.cfg.get('solver', 'shock-capturing', 'none')
        if sc not in ('none', 'entropy-filter', 'artificial-viscosity'):
            raise NotImplementedError(f'Shock capturing {sc!r} is not '
                                      'provided')
        self._av = None
        if self._mpi_inters and sc != 'none':
            raise NotImplementedError('Shock capturing across partitions is '
                                      'not provided')
        if sc == 'artificial-viscosity':
            if self.name != 'navier-stokes':
                raise ValueError('Artificial viscosity needs the '
                                 'Navier-Stokes system')
            from pyfr_gb300.solvers.artvisc import ArtificialViscosity
            self._av = ArtificialViscosity(self, self.cfg)
            av = {et: e.artvisc_fpts for et, e in self.ele_map.items()}
            for i, v in zip(self._sided_inters, self.make_field_views(av)):
                i.artvisc = v[0]

        self.backend.commit()
        for b in self._bc_inters:
            b.bind_device(self._tmat)
        for e in self.ele_map.values():
            e.tmat = self._tmat
        self._gen_kernels()
        if self._av:
            self._av.add_kernels(self._kernels, self._ktags)

        # Shock capturing by the entropy filter
        # (pyfr/solvers/baseadvec/system.py:36-44)
        self._ef = None
        if sc == 'entropy-filter':
            from pyfr_gb300.solvers.entfilter import EntropyFilter
            self._ef = EntropyFilter(self, self.cfg)
            self._ef.add_kernels(self._kernels, self._ktags)

        # Maximum wave speed over each element type
        # (pyfr/solvers/baseadvec/system.py:48-52)
        if self._needs_cfl:
            self._wspd_red_kerns = [
                self.backend.kernel('reduction', 'max', ['x'], {'x': e._wspd})
                for e in self.ele_map.values()]
        self.backend.commit()
        self._graph_cache = {}

        # Host-side geometry and gather maps were only needed to build the
        # kernels
        for e in self.ele_map.values():
            e.release_host_geometry()
        self.backend.release_host_copies()

    def _gen_kernels(self):
        self._kernels = kernels = defaultdict(list)
        self._ktags = {}

        provs = [('eles', list(self.ele_map.values())),
                 ('iint', self._int_inters), ('mpiint', self._mpi_inters),
                 ('bcint', self._bc_inters)]
        for pn, plist in provs:
            for p in plist:
                for kn, kget in p.kernels.items():
                    params = inspect.signature(kget).parameters
                    if 'uin' in params or 'fout' in params:
                        for i in range(self.nrhs):
                            k = kget(i)
                            if isinstance(k, NullKernel):
                                continue
                            key = (f'{pn}/{kn}', i, None) if 'uin' in params \
                                else (f'{pn}/{kn}', None, i)
                            kernels[key].append(k)
                            self._ktags[k] = f'{pn}/{id(p)}'
                    else:
                        k = kget()
                        if isinstance(k, NullKernel):
                            continue
                        kernels[f'{pn}/{kn}', None, None].append(k)
                        self._ktags[k] = f'{pn}/{id(p)}'

    def _get_kernels(self, uinbank, foutbank):
        kernels = defaultdict(list)
        for (kn, ui, fo), k in self._kernels.items():
            if ((ui is None and fo is None) or
                    (ui is not None and ui == uinbank) or
                    (fo is not None and fo == foutbank)):
                kernels[kn].extend(k)
        return kernels

    def _kdeps(self, kdict, kern, *dnames):
        return [k for n in dnames for k in kdict[n]
                if self._ktags[kern] == self._ktags[k]]

    def _group(self, g, kerns, subs=[]):
        kerns = [k for k in kerns if k is not None]
        subs = [[(k, n) for k, n in s if k] for s in subs]
        g.group(kerns, [s for s in subs if len(s) > 1])

    def _rhs_graphs_cached(self, uin, fout):
        key = ('rhs', uin, fout)
        if key not in self._graph_cache:
            gs = self._rhs_graphs(uin, fout)
            if self._mpi_inters:
                gs = self._with_exchanges(gs, uin, fout)
            self._graph_cache[key] = gs
        return self._graph_cache[key]

    # ---- faces shared with other partitions -------------------------------

    def _exchange(self, field):
        """The host step exchanging one field's packed face data with every
        neighbouring partition: device-to-host copies and posted transfers,
        then the received data to the device."""
        lib, be = self.backend.lib, self.backend

        def post(stream):
            if self.exchanger is None:
                raise RuntimeError('Partitions need an exchanger')
            items = []
            for m in self._mpi_inters:
                x, item = m.xchg_items(field)
                lib.memcpy_dtoh(x.hsend.ctypes.data, x.send.data, x.nbytes,
                                stream)
                items.append(item)
            lib.stream_sync(stream)
            self.exchanger.post(items)

        def complete(stream):
            self.exchanger.complete()
            for m in self._mpi_inters:
                x, _ = m.xchg_items(field)
                lib.memcpy_htod(x.recv.data, x.hrecv.ctypes.data, x.nbytes,
                                stream)
            be.wait()

        return HostStep(post, complete, f'xchg_{field}')

    def _mpi_graph(self, kerns):
        g = self.backend.graph()
        g.add_all(kerns)
        g.commit()
        return g

    def _with_exchanges(self, gs, uin, fout):
        """The right-hand side's graphs with the exchanges: after the first
        graph (the solution at the flux points) the packed solution, and
        for Navier-Stokes after the second (the gradient at the flux
        points) the packed gradient; the interface kernels of the shared
        faces run just before the graph that reads their results
        (pyfr/solvers/baseadvec/system.py:58-136,
        pyfr/solvers/baseadvecdiff/system.py:54-231)."""
        k = self._get_kernels(uin, fout)
        out = [gs[0], self._mpi_graph(k['mpiint/scal_pack']),
               self._exchange('scal')]
        if len(gs) == 2:
            out += [self._mpi_graph(k['mpiint/comm_flux']), gs[1]]
        else:
            out += [self._mpi_graph(k['mpiint/con_u']), gs[1],
                    self._mpi_graph(k['mpiint/vect_pack']),
                    self._exchange('vect'),
                    self._mpi_graph(k['mpiint/comm_flux']), *gs[2:]]
        return tuple(out)

    def rhs_phases(self, t, uinbank, foutbank):
        """The right-hand side as a list of callables, each exchange split
        into its post and its completion, for driving several partitions
        of one process in lockstep."""
        stream = self.backend.stream
        phases = []
        if self.time_dependent:
            phases.append(lambda: self.set_time(t))
        for k in self.prepare_kernels(uinbank, t):
            phases.append(lambda k=k: k.run(stream))
        for g in self._rhs_graphs_cached(uinbank, foutbank):
            if isinstance(g, HostStep):
                phases.extend(lambda k=k: k.run(stream) for k in g.klist)
            else:
                phases.append(lambda g=g: self.backend.run_graph(g))
        return phases

    def rhs_graphs(self, uinbank, foutbank):
        return self._rhs_graphs_cached(uinbank, foutbank)

    @property
    def time_dependent(self):
        """Whether a boundary value or a source term depends on the
        time."""
        return (any(getattr(b, 'time_dependent', False)
                    for b in self._bc_inters) or
                any(e.src_uses_t for e in self.ele_map.values()))

    @property
    def controlled_bcs(self):
        """The controllers of the controlled characteristic boundaries."""
        return [b.controller for b in self._bc_inters
                if getattr(b, 'controller', None) is not None]

    def prepare_kernels(self, ubank, t):
        """Host steps before a right-hand side at time t from bank ubank:
        the boundary controllers (pyfr/solvers/base/system.py:408-415).
        They read the solution on the host, so they run outside captured
        graphs."""
        ctrls = self.controlled_bcs
        if not ctrls:
            return []

        def solns():
            return dict(zip(self.ele_types, self.ele_scal_upts(ubank)))

        def run(stream):
            for c in ctrls:
                c.prepare(solns, t, stream)

        return [Kernel(run, name='bcprepare')]

    @property
    def has_src_macros(self):
        return any(e.has_src_macros for e in self.ele_map.values())

    def evalsrcmacros(self, uinoutbank):
        """Overwrite a bank with the source terms evaluated from it
        (pyfr/solvers/base/system.py:478-481)."""
        k = self._get_kernels(uinoutbank, None)['eles/evalsrcmacros']
        self.backend.run_kernels(k, wait=True)

    def _add_src(self, g, k, deps):
        """The source terms after a fused divergence apply."""
        for l in k['eles/addsrc']:
            g.add(l, deps=deps(l, 'eles/tdivtconf_cat'))

    def set_time(self, t):
        """Set the stage time read by the boundary values (an RHS called
        outside an integrator step)."""
        self._tmat.set(np.array([[t, t]]))

    def stage_time_kernel(self, c, dt=None, dt_dev=None):
        """A kernel setting the stage time t0 + c*dt, dt from device
        memory (``dt_dev``) or the given value."""
        lib, tm = self.backend.lib, self._tmat
        dp = dt_dev.data if dt_dev is not None else None

        def run(stream):
            lib.stage_time(tm.data, dp, float(dt or 0.0), float(c), stream)

        return Kernel(run, mats=[tm] + ([dt_dev] if dt_dev is not None
                                        else []), name='stage_time')

    def rhs(self, t, uinbank, foutbank):
        if uinbank >= self.nrhs or foutbank >= self.nrhs:
            raise ValueError('Invalid register numbers')
        if self.time_dependent:
            self.set_time(t)
        for k in self.prepare_kernels(uinbank, t):
            k.run(self.backend.stream)
        for g in self._rhs_graphs_cached(uinbank, foutbank):
            self.backend.run_graph(g)

    def preproc_kernels(self, uinbank):
        """Before the first step: filter, then every element's and face's
        minimum entropy (pyfr/solvers/baseadvec/entfilter.py:160-194)."""
        if not self._ef:
            return []
        k = self._get_kernels(uinbank, None)
        return (k['eles/entropy_filter'] + k['eles/local_entropy'] +
                k['eles/disu'] + k['iint/comm_entropy'] +
                k['bcint/comm_entropy'])

    def postproc_kernels(self, uinbank):
        """After every step: filter the new solution."""
        if not self._ef:
            return []
        return self._get_kernels(uinbank, None)['eles/entropy_filter']

    def compute_max_wavespeed(self, uinbank):
        """Largest element wave speed of the solution in bank uinbank
        (pyfr/solvers/baseadvec/system.py:157-161)."""
        k = self._get_kernels(uinbank, None)
        self.backend.run_kernels(k['eles/wavespeed'] + self._wspd_red_kerns,
                                 wait=True)
        return max(k.retval[0] for k in self._wspd_red_kerns)

    def ele_scal_upts(self, idx):
        return [eb[idx].get() for eb in self.ele_banks]

    def set_ele_scal_upts(self, idx, arrs):
        for eb, a in zip(self.ele_banks, arrs):
            eb[idx].set(a)


class EulerSystem(BaseSystem):
    name = 'euler'
    elementscls = EulerElements
    intinterscls = EulerIntInters
    mpiinterscls = EulerMPIInters
    bcinterscls = EulerBCInters

    def _rhs_graphs(self, uinbank, foutbank):
        k = self._get_kernels(uinbank, foutbank)

        def deps(dk, *names):
            return self._kdeps(k, dk, *names)

        g_intf = self.backend.graph()
        # (with the entropy filter: filter the input first, then exchange
        # the new face minima; pyfr/solvers/baseadvec/system.py:58-90;
        # source terms of the solution read a copy of it)
        g_intf.add_all(k['eles/entropy_filter'])
        for l in k['eles/copy_soln']:
            g_intf.add(l, deps=deps(l, 'eles/entropy_filter'))
        for l in k['eles/disu']:
            g_intf.add(l, deps=deps(l, 'eles/entropy_filter'))
        g_intf.add_all(k['iint/comm_entropy'], deps=k['eles/entropy_filter'])
        g_intf.add_all(k['bcint/comm_entropy'],
                       deps=k['eles/disu'] + k['iint/comm_entropy'])
        g_intf.add_all(k['iint/comm_flux'], deps=k['eles/disu'])
        g_intf.add_all(k['bcint/comm_flux'],
                       deps=k['eles/disu'] + k['bcint/comm_entropy'])
        g_intf.commit()

        g_flux_div = self.backend.graph()
        # (flux anti-aliasing: the solution at the quadrature points first)
        g_flux_div.add_all(k['eles/qptsu'])
        for l in k['eles/tdisf']:
            g_flux_div.add(l, deps=deps(l, 'eles/qptsu'))
        if k['eles/tdivtconf_cat']:
            # Fused divergence, correction and negdivconf
            for l in k['eles/tdivtconf_cat']:
                g_flux_div.add(l, deps=deps(l, 'eles/tdisf'))
            self._add_src(g_flux_div, k, deps)
            g_flux_div.commit()
            return g_intf, g_flux_div

        for l in k['eles/tdivtpcorf']:
            g_flux_div.add(l, deps=deps(l, 'eles/tdisf'))
        for l in k['eles/tdivtconf']:
            g_flux_div.add(l, deps=deps(l, 'eles/tdivtpcorf'))
        for l in k['eles/negdivconf']:
            g_flux_div.add(l, deps=deps(l, 'eles/tdivtconf'))

        kgroup = [k['eles/tdisf'], k['eles/tdivtpcorf'], k['eles/tdivtconf'],
                  k['eles/negdivconf']]
        for ks in zip_longest(*kgroup):
            self._group(g_flux_div, ks, subs=[[(ks[0], 'f'), (ks[1], 'b')]])
        g_flux_div.commit()

        return g_intf, g_flux_div


class NavierStokesSystem(BaseSystem):
    name = 'navier-stokes'
    elementscls = NavierStokesElements
    intinterscls = NavierStokesIntInters
    mpiinterscls = NavierStokesMPIInters
    bcinterscls = NavierStokesBCInters

    def __init__(self, *args, **kwargs):
        super().__init__(*args, **kwargs)
        self._setup_face_gradients()

    def _setup_face_gradients(self):
        """With single-precision state and every element affine, the flux
        kernel leaves the corrected gradient in reference space instead of
        storing its transform (one field write per right-hand side less),
        the face gradients are interpolated from it, and the interface
        kernel transforms them with the elements' metric terms (an affine
        transform commutes with the interpolation).  ``[backend-b200]
        face-gradients = auto`` (this when the conditions hold) or
        ``physical`` (the reference's order: transform at the points)."""
        be, cfg = self.backend, self.cfg
        opt = cfg.get('backend-b200', 'face-gradients', 'auto')
        if opt not in ('auto', 'physical'):
            raise ValueError('face-gradients must be auto or physical')
        if opt == 'physical' or be.fpdtype != np.float32 or \
                self._bc_inters or self._mpi_inters or \
                cfg.get('solver', 'shock-capturing', 'none') != 'none' or \
                any(e.antialias for e in self.ele_map.values()):
            return
        mets = []
        for e in self.ele_map.values():
            m = e.affine_metrics()
            if m is None:
                return
            mets.append(m)
        nd = self.ndims
        ncol = sum(len(r) for _, r in mets)
        if ncol >= 2**31:
            return
        emet = np.empty((nd*nd + 1, ncol))
        col = 0
        for e, (sm, rj) in zip(self.ele_map.values(), mets):
            n = len(rj)
            emet[:nd*nd, col:col + n] = sm.reshape(nd*nd, n)
            emet[nd*nd, col:col + n] = rj
            e.face_metric_col = col
            e.grad_writeback = False
            col += n
        mat = be.const_matrix(emet, tags={'align'})
        for i in self._int_inters:
            i.set_face_metrics(mat)
        be.commit()

    def _rhs_graphs(self, uinbank, foutbank):
        k = self._get_kernels(uinbank, foutbank)

        def deps(dk, *names):
            return self._kdeps(k, dk, *names)

        # Graph 1: solution at the flux points and the common solution
        g_soln = self.backend.graph()
        g_soln.add_all(k['eles/entropy_filter'])
        for l in k['eles/copy_soln']:
            g_soln.add(l, deps=deps(l, 'eles/entropy_filter'))
        for l in k['eles/disu']:
            g_soln.add(l, deps=deps(l, 'eles/entropy_filter'))
        g_soln.add_all(k['iint/comm_entropy'], deps=k['eles/entropy_filter'])
        g_soln.add_all(k['bcint/comm_entropy'],
                       deps=k['eles/disu'] + k['iint/comm_entropy'])
        for l in k['eles/copy_fpts']:
            g_soln.add(l, deps=deps(l, 'eles/disu'))
        kdeps = k['eles/copy_fpts'] or k['eles/disu']
        g_soln.add_all(k['iint/con_u'], deps=kdeps)
        g_soln.add_all(k['bcint/con_u'], deps=kdeps)
        # Artificial viscosity: zero the vertex values, sense every
        # element, then fill the point values once all sensors are done
        # (pyfr/solvers/baseadvecdiff/artvisc.py:246-264)
        g_soln.add_all(k['vtx/vtx_zero'])
        g_soln.add_all(k['eles/shocksensor'], deps=k['vtx/vtx_zero'])
        g_soln.add_all(k['eles/avfill'], deps=k['eles/shocksensor'])
        g_soln.commit()

        if k['eles/qptsu']:
            return (g_soln,) + self._rhs_graphs_antialias(k, deps)
        if k['eles/tgradcoru_upts_cat']:
            return (g_soln,) + self._rhs_graphs_fused(k, deps)

        # Graph 2: corrected gradient, fused flux, face gradients, common
        # flux and the divergence of the partially corrected flux
        g_grad_flux = self.backend.graph()
        g_grad_flux.add_all(k['eles/tgradpcoru_upts'])
        for l in k['eles/tgradcoru_upts']:
            g_grad_flux.add(l, deps=deps(l, 'eles/tgradpcoru_upts'))
        for l in k['eles/tdisf_fused']:
            g_grad_flux.add(l, deps=deps(l, 'eles/tgradcoru_upts'))
        for l in k['eles/gradcoru_fpts']:
            g_grad_flux.add(l, deps=deps(l, 'eles/tdisf_fused'))
        g_grad_flux.add_all(k['iint/comm_flux'], deps=k['eles/gradcoru_fpts'])
        g_grad_flux.add_all(k['bcint/comm_flux'], deps=k['eles/gradcoru_fpts'])
        for l in k['eles/tdivtpcorf']:
            g_grad_flux.add(l, deps=deps(l, 'eles/tdisf_fused'))

        kgroup = [k['eles/tgradpcoru_upts'], k['eles/tgradcoru_upts'],
                  k['eles/tdisf_fused'], k['eles/gradcoru_fpts'],
                  k['eles/tdivtpcorf']]
        for ks in zip_longest(*kgroup):
            self._group(g_grad_flux, ks, subs=[
                [(ks[0], 'out'), (ks[1], 'out'), (ks[2], 'gradu'),
                 (ks[3], 'b')],
                [(ks[2], 'f'), (ks[4], 'b')],
            ])
        g_grad_flux.commit()

        # Graph 3: correction and physical divergence
        g_div = self.backend.graph()
        g_div.add_all(k['eles/tdivtconf'])
        for l in k['eles/negdivconf']:
            g_div.add(l, deps=deps(l, 'eles/tdivtconf'))
        for k1, k2 in zip_longest(k['eles/tdivtconf'], k['eles/negdivconf']):
            self._group(g_div, [k1, k2])
        g_div.commit()

        return g_soln, g_grad_flux, g_div

    def _rhs_graphs_antialias(self, k, deps):
        """Graphs 2 and 3 with flux anti-aliasing
        (pyfr/solvers/baseadvecdiff/system.py:107-200 without gradient
        fusion): the corrected gradient, transformed in place to physical
        space, goes to the flux points and to the quadrature points, where
        the flux is evaluated with the interpolated solution; the
        divergence projects it back with M9."""
        g = self.backend.graph()
        if k['eles/tgradcoru_upts_cat']:
            g.add_all(k['eles/tgradcoru_upts_cat'])
            gdeps = 'eles/tgradcoru_upts_cat'
        else:
            g.add_all(k['eles/tgradpcoru_upts'])
            for l in k['eles/tgradcoru_upts']:
                g.add(l, deps=deps(l, 'eles/tgradpcoru_upts'))
            gdeps = 'eles/tgradcoru_upts'
        for l in k['eles/gradcoru_u']:
            g.add(l, deps=deps(l, gdeps))
        for l in k['eles/gradcoru_fpts']:
            g.add(l, deps=deps(l, 'eles/gradcoru_u'))
        for l in k['eles/gradcoru_qpts']:
            g.add(l, deps=deps(l, 'eles/gradcoru_u'))
        g.add_all(k['eles/qptsu'])
        g.add_all(k['iint/comm_flux'], deps=k['eles/gradcoru_fpts'])
        g.add_all(k['bcint/comm_flux'], deps=k['eles/gradcoru_fpts'])
        for l in k['eles/tdisf']:
            g.add(l, deps=deps(l, 'eles/gradcoru_qpts', 'eles/qptsu'))
        for l in k['eles/tdivtpcorf']:
            g.add(l, deps=deps(l, 'eles/tdisf'))
        g.commit()

        g_div = self.backend.graph()
        if k['eles/tdivtconf_cat']:
            g_div.add_all(k['eles/tdivtconf_cat'])
            self._add_src(g_div, k, deps)
        else:
            g_div.add_all(k['eles/tdivtconf'])
            for l in k['eles/negdivconf']:
                g_div.add(l, deps=deps(l, 'eles/tdivtconf'))
        g_div.commit()
        return g, g_div

    def _rhs_graphs_fused(self, k, deps):
        """Graphs 2 and 3 with fused operator applies: the corrected
        gradient in one apply, the face gradients in one launch, and the
        divergence, correction and negdivconf in one apply (which then
        waits for the common flux)."""
        g_grad_flux = self.backend.graph()
        g_grad_flux.add_all(k['eles/tgradcoru_upts_cat'])
        for l in k['eles/tdisf_fused']:
            g_grad_flux.add(l, deps=deps(l, 'eles/tgradcoru_upts_cat'))
        for l in k['eles/gradcoru_fpts']:
            g_grad_flux.add(l, deps=deps(l, 'eles/tdisf_fused'))
        g_grad_flux.add_all(k['iint/comm_flux'], deps=k['eles/gradcoru_fpts'])
        g_grad_flux.add_all(k['bcint/comm_flux'], deps=k['eles/gradcoru_fpts'])
        g_grad_flux.commit()

        g_div = self.backend.graph()
        g_div.add_all(k['eles/tdivtconf_cat'])
        self._add_src(g_div, k, deps)
        g_div.commit()
        return g_grad_flux, g_div

    def _compute_grads_graph(self, uinbank):
        key = ('grads', uinbank)
        if key in self._graph_cache:
            return self._graph_cache[key]

        k = self._get_kernels(uinbank, None)

        def deps(dk, *names):
            return self._kdeps(k, dk, *names)

        g = self.backend.graph()
        g.add_all(k['eles/disu'])
        for l in k['eles/copy_fpts']:
            g.add(l, deps=deps(l, 'eles/disu'))
        kdeps = k['eles/copy_fpts'] or k['eles/disu']
        g.add_all(k['iint/con_u'], deps=kdeps)
        if k['eles/tgradcoru_upts_cat']:
            g.add_all(k['eles/tgradcoru_upts_cat'], deps=k['iint/con_u'])
            for l in k['eles/gradcoru_u']:
                g.add(l, deps=deps(l, 'eles/tgradcoru_upts_cat'))
        else:
            g.add_all(k['eles/tgradpcoru_upts'], deps=k['iint/con_u'])
            for l in k['eles/tgradcoru_upts']:
                g.add(l, deps=deps(l, 'eles/tgradpcoru_upts') + k['iint/con_u'])
            for l in k['eles/gradcoru_u']:
                g.add(l, deps=deps(l, 'eles/tgradcoru_upts'))
        g.commit()

        self._graph_cache[key] = (g,)
        return (g,)

    def compute_grads(self, t, uinbank):
        for g in self._compute_grads_graph(uinbank):
            self.backend.run_graph(g)

    def grad_upts(self):
        """Physical gradients (ndims, nupts, nvars, neles) per element type
        after ``compute_grads``."""
        return [e._grad_upts.get() for e in self.ele_map.values()]


SYSTEMS = {'euler': EulerSystem, 'navier-stokes': NavierStokesSystem}
