"""Controlled characteristic boundaries: ``char-riem-inv-mass-flow`` and
``char-riem-inv-pressure`` (pyfr/solvers/euler/inters.py:108-294).

The ghost state is that of ``char-riem-inv`` with the free-stream pressure
replaced by p(t) = ic + im*t (pyfr/solvers/euler/kernels/bcs/
char-riem-inv-controlled.mako).  Before every right-hand side a host
controller (``prepare``, the reference's ``ControlledBCMixin.prepare``)
counts the evaluations; every ``nsteps`` of them (and until it has a
previous time) it measures the boundary's mass flow, or its area-averaged
pressure, from the right-hand side's input solution with a surface
quadrature (pyfr/quadrules/surface.py:8-51), relaxes the measurement into
a running average and moves the pressure interpolation towards the target.
The interpolation coefficients (ic, im) live in device memory, where the
boundary kernels read them with the stage time.
"""

import ctypes as C
import weakref

import numpy as np

from pyfr_gb300.shapes import _proj


def _face_rule(cfg, cfgsect, kind):
    """Points (in face coordinates) and weights of the surface quadrature
    of one face kind: ``quad-pts-<kind>`` (a rule name or a literal rule)
    or the interfaces' flux-point rule, of the smallest size exact for
    ``quad-deg-<kind>`` (or ``quad-deg``), the selection of
    pyfr/quadrules/__init__.py:44-78."""
    from pyfr_gb300.quadrules import parse_rule, tensor_rule

    rname = cfg.get(f'solver-interfaces-{kind}', 'flux-pts', 'gauss-legendre')
    qrule = cfg.get(cfgsect, f'quad-pts-{kind}', rname)
    nd = {'line': 1, 'quad': 2, 'tri': 2}[kind]
    if not qrule.replace('-', '').replace('~', '').isalnum():
        pts, wts = parse_rule(qrule, nd)
        if wts is None:
            raise ValueError(f'{cfgsect}: the surface rule needs weights')
        return np.asarray(pts, dtype=float).reshape(len(wts), nd), wts
    if cfg.hasopt(cfgsect, f'quad-deg-{kind}'):
        qdeg = cfg.getint(cfgsect, f'quad-deg-{kind}')
    else:
        qdeg = cfg.getint(cfgsect, 'quad-deg')
    if kind == 'tri' or qrule not in ('gauss-legendre',
                                      'gauss-legendre-lobatto'):
        raise NotImplementedError(f'{cfgsect}: surface rule {qrule!r} on '
                                  f'{kind} faces is not provided')
    # Gauss-Legendre with n points is exact to degree 2n - 1,
    # Gauss-Legendre-Lobatto to 2n - 3
    if qrule == 'gauss-legendre':
        n = max(1, -(-(qdeg + 1)//2))
    else:
        n = max(2, -(-(qdeg + 3)//2))
    pts, wts = tensor_rule(qrule, n, nd)
    return pts.reshape(len(wts), nd), wts


class SurfaceIntegrator:
    """Interpolation to, weights of, and scaled normals at the surface
    quadrature points of every face of a boundary."""

    def __init__(self, cfg, cfgsect, elemap, side):
        self.m0, self.qwts, self.eidxs, self.norms = {}, {}, {}, {}
        etypes = np.asarray(side.etypes)
        eidxs, fidxs = np.asarray(side.eidxs), np.asarray(side.fidxs)
        for key in sorted({(str(t), int(f)) for t, f in zip(etypes, fidxs)}):
            etype, fidx = key
            mask = (etypes == etype) & (fidxs == fidx)
            eles = elemap[etype]
            kind, proj, norm = eles.basis.faces[fidx]
            fpts, wts = _face_rule(cfg, cfgsect, kind)
            ppts = _proj(proj, fpts)
            s, _ = eles.smats_djac_at_np(ppts)         # (p, l, k, e)
            ei = eidxs[mask]
            pn = np.einsum('plke,l->pek', s[..., ei],
                           np.asarray(norm, dtype=float))
            self.m0[key] = eles.basis.ubasis.nodal_basis_at(ppts)
            self.qwts[key] = wts
            self.eidxs[key] = ei
            self.norms[key] = pn.transpose(2, 0, 1)    # (ndims, p, n)

    def interp(self, solns):
        """(solution at the points (nvars, npts, n), weights, normals) of
        each face group, from the solution at the solution points of every
        element type."""
        for key, m0 in self.m0.items():
            u = solns[key[0]][:, :, self.eidxs[key]]
            nupts, nvars, n = u.shape
            uf = (m0 @ u.reshape(nupts, -1)).reshape(-1, nvars, n)
            yield uf.swapaxes(0, 1), self.qwts[key], self.norms[key]


class ControlledBC:
    """The host controller of one controlled boundary; ``kind`` is
    'mass-flow' or 'pressure'."""

    def __init__(self, be, cfg, cfgsect, elemap, side, kind, con_to_pri):
        from pyfr_gb300.solvers.elements import npeval

        self.be, self.cfg, self.cfgsect, self.kind = be, cfg, cfgsect, kind
        self.con_to_pri = con_to_pri
        consts = cfg.items_as('constants', float)

        def ev(k):
            return float(npeval(cfg.getexpr(cfgsect, k), dict(consts)))

        tkey = 'mass-flow-rate' if kind == 'mass-flow' else 'pressure'
        self.target, self.alpha, self.eta = ev(tkey), ev('alpha'), ev('eta')
        self.tstart = cfg.getfloat(cfgsect, 'tstart', 0.0)
        self.nsteps = cfg.getint(cfgsect, 'nsteps', 100)
        self.surf = SurfaceIntegrator(cfg, cfgsect, elemap, side)

        if kind == 'mass-flow':
            self._qn = [self.surf.norms[k]*self.surf.qwts[k][:, None]
                        for k in self.surf.m0]
            default_c = ev('p')
        else:
            self._qnmag = [np.sqrt(np.einsum('hij,hij->ij', n, n))*w[:, None]
                           for n, w in ((self.surf.norms[k], self.surf.qwts[k])
                                        for k in self.surf.m0)]
            self.area = float(sum(q.sum() for q in self._qnmag))
            default_c = self.target

        self.interp_c, self.interp_m = default_c, 0.0
        self.meas_avg, self.tprev, self.nstep_counter = 0.0, None, 0
        self.history = []

        # (t, measured average, new pressure) of every update to a CSV
        # file with the 'file' option, flushed every 'flushsteps' lines
        self._csv = None
        if cfg.hasopt(cfgsect, 'file'):
            self._csv = open(cfg.get(cfgsect, 'file'), 'w')
            self._csv_flush = cfg.getint(cfgsect, 'flushsteps', 10)
            print('t,mf,pbc' if kind == 'mass-flow' else 't,p,pbc',
                  file=self._csv)
            weakref.finalize(self, self._csv.close)

        # (ic, im) in device memory, staged through page-locked memory
        self.ctrl = be.matrix((1, 2), dtype=np.float64)
        be.commit()
        self._host = C.c_void_p()
        be.lib.host_alloc(C.byref(self._host), 16)
        weakref.finalize(self, be.lib.host_free, self._host.value)
        self._evt = C.c_void_p()
        be.lib.event_create(C.byref(self._evt))
        weakref.finalize(self, be.lib.event_destroy, self._evt.value)
        self._pending, self._sent = False, None
        self.upload(be.stream)

    def upload(self, stream):
        """Enqueue the copy of (ic, im) to device memory when changed."""
        vals = (self.interp_c, self.interp_m)
        if vals == self._sent:
            return
        lib = self.be.lib
        if self._pending:
            lib.event_sync(self._evt.value)
        (C.c_double*2).from_address(self._host.value)[:] = vals
        lib.memcpy_htod(self.ctrl.data, self._host.value, 16, stream)
        lib.event_record(self._evt.value, stream)
        self._pending, self._sent = True, vals

    def _measure(self, solns):
        if self.kind == 'mass-flow':
            return float(sum(np.einsum('hij,hij', u[1:-1], qn) for
                             (u, _, _), qn in zip(self.surf.interp(solns),
                                                  self._qn)))
        pnum = 0.0
        for (u, _, _), qm in zip(self.surf.interp(solns), self._qnmag):
            p = self.con_to_pri(list(u), self.cfg)[-1]
            pnum += float(np.einsum('ij,ij', p, qm))
        return pnum/self.area

    def _correction(self, p0, dt):
        if self.kind == 'mass-flow':
            return p0 + dt*self.eta*(1 - self.target/self.meas_avg)
        return p0 + dt*self.eta*(self.target - self.meas_avg)

    def prepare(self, solns_fn, t, stream):
        """Before the right-hand side at time t whose input solution
        ``solns_fn()`` returns ({etype: (nupts, nvars, neles)})."""
        update = self.nstep_counter % self.nsteps == 0
        if (update or not self.tprev) and t >= self.tstart:
            meas = self._measure(solns_fn())
            if not self.tprev:
                self.meas_avg = meas
                self.tprev = t
            else:
                a = self.alpha
                self.meas_avg = a*meas + (1 - a)*self.meas_avg
                dt = t - self.tprev
                self.tprev = t
                p0 = self.interp_m*t + self.interp_c
                p1 = self._correction(p0, dt)
                self.interp_m = (p1 - p0)/dt
                self.interp_c = p0 - self.interp_m*t
                self.history.append((t, self.meas_avg, p1))
                if self._csv:
                    print(f'{t},{self.meas_avg},{p1}', file=self._csv)
                    if len(self.history) % self._csv_flush == 0:
                        self._csv.flush()
        self.upload(stream)
        self.nstep_counter += 1

    def state(self):
        """The controller state (the reference serialises the same five
        values, pyfr/solvers/euler/inters.py:196-203)."""
        return (self.interp_c, self.interp_m, self.meas_avg,
                self.tprev or 0, self.nstep_counter)
