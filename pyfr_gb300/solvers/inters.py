"""Interior interfaces of the Euler and Navier-Stokes systems.

Builds the left/right gather views over the flux-point fields and the
scaled left normals, with the reference's memory-access permutation (all
interface arrays ordered by the left side's flux-point address,
``pyfr/solvers/base/inters.py:70-90``,
``pyfr/solvers/baseadvec/inters.py:8-28``), and declares the interface
kernels (``pyfr/solvers/euler/inters.py:28-38``,
``pyfr/solvers/navstokes/inters.py:29-48``).
"""

import ctypes as C

import numpy as np


def inter_arrays(side, meth, elemap, perm=Ellipsis):
    """Concatenate the per-(etype, face) arrays of ``meth`` in interface
    order, then apply ``perm``."""
    parts, reorder = [], []
    for etype, fidx, eidxs, idx in side.foreach():
        parts.append(getattr(elemap[etype], meth)(eidxs, fidx))
        reorder.append(np.repeat(idx, elemap[etype].nfacefpts[fidx]))

    if not parts:
        return []

    ro = np.argsort(np.concatenate(reorder), kind='stable')[perm]
    return [np.concatenate(a)[ro] for a in zip(*parts)]


def field_view_arrays(side, field, elemap):
    """(matmap, rowmap, colmap) of a flux-point field over one side."""
    matmap, rowmap, colmap, reorder = [], [], [], []
    for etype, fidx, eidxs, idx in side.foreach():
        mat, eles = field[etype], elemap[etype]
        fpts = eles.srtd_face_fpts[fidx][eidxs]
        nfp = fpts.shape[1]
        matmap.append(np.full(len(eidxs)*nfp, mat.mid))
        rowmap.append(fpts.ravel())
        colmap.append(np.repeat(eidxs, nfp))
        reorder.append(np.repeat(idx, nfp))

    ro = np.argsort(np.concatenate(reorder), kind='stable')
    return (np.concatenate(matmap)[ro], np.concatenate(rowmap)[ro],
            np.concatenate(colmap)[ro])


class BaseIntInters:
    # Set by the system: every flux point lies on an interior interface
    covers = False

    def __init__(self, be, lhs, rhs, elemap, cfg):
        self._be = be
        self.elemap = elemap
        self.cfg = cfg
        self.lhs, self.rhs = lhs, rhs

        first = next(iter(elemap.values()))
        self.ndims, self.nvars = first.ndims, first.nvars
        self.ninters = len(lhs)
        self.ninterfpts = sum(elemap[et].nfacefpts[fi]*len(ei)
                              for et, fi, ei in lhs.items())

        self.c = cfg.items_as('constants', float)
        self.kernels = {}

        # Order all interface arrays by the left side's flux-point address
        scal = {t: e._scal_fpts for t, e in elemap.items()}
        self._perm = self._perm_for_field(self._perm_side(), scal)
        self._pnorm_lhs = self._const_mat(lhs, 'get_pnorms_for_inters')

    def _perm_side(self):
        return self.lhs

    def _perm_for_field(self, side, field):
        m, r, c = field_view_arrays(side, field, self.elemap)
        v = self._be.view(m, r, c, vshape=())
        return np.argsort(v.mapping._host[0], kind='stable')

    def _const_mat(self, side, meth):
        m = inter_arrays(side, meth, self.elemap, self._perm)
        m = m[0] if m else np.empty((0, self.ndims))
        return self._be.const_matrix(np.atleast_2d(m.T))

    def _view(self, side, meth, vshape=()):
        vm = inter_arrays(side, meth, self.elemap, self._perm)
        return self._be.view(*vm, vshape=vshape)

    def _scal_view(self, side, meth):
        return self._view(side, meth, (self.nvars,))

    def _vect_view(self, side, meth):
        return self._view(side, meth, (self.ndims, self.nvars))


def riemann_p_min(cfg, be):
    """Star-pressure floor of the exact Riemann solver: the entropy
    filter's p-min when it is on, else [solver-interfaces] p-min
    (pyfr/solvers/euler/inters.py:12-25)."""
    if cfg.get('solver', 'shock-capturing', 'none') == 'entropy-filter':
        return cfg.getfloat('solver-entropy-filter', 'p-min', 1e-6)
    return cfg.getfloat('solver-interfaces', 'p-min', 5*be.fpdtype_eps)


class EulerIntInters(BaseIntInters):
    def __init__(self, *args, **kwargs):
        super().__init__(*args, **kwargs)

        rsolver = self.cfg.get('solver-interfaces', 'riemann-solver')
        p_min = riemann_p_min(self.cfg, self._be)
        self._tplargs = dict(ndims=self.ndims, nvars=self.nvars,
                             rsolver=rsolver, c=self.c, p_min=p_min)

        self._be.pointwise.register('pyfr.solvers.euler.kernels.intcflux')
        self.kernels['comm_flux'] = lambda: self._be.kernel(
            'intcflux', tplargs=self._tplargs, dims=[self.ninterfpts],
            ul=self.scal_lhs, ur=self.scal_rhs, nl=self._pnorm_lhs)


class NavierStokesIntInters(BaseIntInters):
    def __init__(self, be, lhs, rhs, elemap, cfg):
        self.cfg = cfg
        super().__init__(be, lhs, rhs, elemap, cfg)

        self._vect_lhs = self._vect_view(lhs, 'get_vect_fpts_for_inters')
        self._vect_rhs = self._vect_view(rhs, 'get_vect_fpts_for_inters')
        self._comm_lhs = self._scal_view(lhs, 'get_comm_fpts_for_inters')
        self._comm_rhs = self._scal_view(rhs, 'get_comm_fpts_for_inters')

        self.c |= cfg.items_as('solver-interfaces', float)

        rsolver = cfg.get('solver-interfaces', 'riemann-solver')
        visc_corr = cfg.get('solver', 'viscosity-correction', 'none')
        p_min = riemann_p_min(cfg, self._be)
        sc = cfg.get('solver', 'shock-capturing', 'none')
        self._tplargs = dict(ndims=self.ndims, nvars=self.nvars,
                             rsolver=rsolver, visc_corr=visc_corr,
                             shock_capturing=sc, c=self.c, p_min=p_min)
        # (the view of the artificial viscosity of the left side, set by
        # the system when shock capturing is artificial viscosity)
        self.artvisc = None
        # (metric matrix and element columns of both sides when the face
        # gradients stay in reference space: set_face_metrics)
        self.facemet = None

        be = self._be
        be.pointwise.register('pyfr.solvers.navstokes.kernels.intconu')
        be.pointwise.register('pyfr.solvers.navstokes.kernels.intcflux')

        self.kernels['con_u'] = lambda: be.kernel(
            'intconu', tplargs=self._tplargs | {'both_sides': self.covers},
            dims=[self.ninterfpts],
            ulin=self.scal_lhs, urin=self.scal_rhs,
            ulout=self._comm_lhs, urout=self._comm_rhs)
        self.kernels['comm_flux'] = lambda: be.kernel(
            'intcflux', tplargs=self._tplargs, dims=[self.ninterfpts],
            ul=self.scal_lhs, ur=self.scal_rhs,
            gradul=self._vect_lhs, gradur=self._vect_rhs, nl=self._pnorm_lhs,
            **({'artvisc': self.artvisc} if self.artvisc is not None else {}),
            **({'facemet': self.facemet} if self.facemet is not None else {}))

    def set_face_metrics(self, emet):
        """The face gradients reach the interface kernel in reference
        space: ``emet`` is the backend matrix of the affine elements'
        metric terms (one column per element, each type from its
        ``face_metric_col``)."""
        cols = [self._be.const_matrix(
            inter_arrays(side, 'get_eidx_for_inters', self.elemap,
                         self._perm)[0][None, :], dtype=np.int32)
            for side in (self.lhs, self.rhs)]
        self.facemet = (emet, *cols)

    def _perm_side(self):
        # For beta = -1/2 order by the right side instead
        # (pyfr/solvers/baseadvecdiff/inters.py:21-28)
        beta = self.cfg.getfloat('solver-interfaces', 'ldg-beta')
        return self.lhs if beta != -0.5 else self.rhs


# ---------------------------------------------------------------------------
# Interfaces with another partition (pyfr/solvers/baseadvec/inters.py:31-47,
# pyfr/solvers/baseadvecdiff/inters.py:33-60, pyfr/solvers/euler/
# inters.py:40-49, pyfr/solvers/navstokes/inters.py:50-66)
# ---------------------------------------------------------------------------

class _Xchg:
    """Exchange buffers of one field over the shared faces: what this side
    packs (send), what it receives (recv) and a scratch target (junk) for
    the other side's outputs of the two-sided interface kernels, all of
    io-shape (nrow, nvars, n); views of recv and junk read them point by
    point; host copies for the transfer."""

    def __init__(self, be, nrow, nvars, n):
        shape = (nrow, nvars, n)
        self.send, self.recv, self.junk = (
            be.matrix(shape, tags={'align'}) for _ in range(3))
        vshape = (nvars,) if nrow == 1 else (nrow, nvars)

        def ident(m):
            return be.view([m.mid]*n, [0]*n, np.arange(n),
                           *([[1]*n] if nrow > 1 else []), vshape=vshape)

        self.rview, self.jview = ident(self.recv), ident(self.junk)
        nb = self.send.nrow*self.send.leaddim*self.send.itemsize
        self.nbytes = nb
        self.hsend = np.empty(nb, dtype=np.uint8)
        self.hrecv = np.empty(nb, dtype=np.uint8)


class BaseMPIInters(BaseIntInters):
    """The faces shared with partition ``rhsrank``: the local side, whose
    views keep the shared face order (no reordering, so that the packed
    data of both partitions line up), the exchange buffers, and the
    interface kernels with the received data as their right side."""

    def __init__(self, be, lhs, rhsrank, elemap, cfg, rank):
        self._be = be
        self.elemap = elemap
        self.cfg = cfg
        self.lhs, self.rhs = lhs, None
        self.rhsrank, self.rank = rhsrank, rank

        first = next(iter(elemap.values()))
        self.ndims, self.nvars = first.ndims, first.nvars
        self.ninters = len(lhs)
        self.ninterfpts = sum(elemap[et].nfacefpts[fi]*len(ei)
                              for et, fi, ei in lhs.items())
        self.c = cfg.items_as('constants', float)
        self.kernels = {}
        self._perm = np.arange(self.ninterfpts)
        self._pnorm_lhs = self._const_mat(lhs, 'get_pnorms_for_inters')
        self._xs = _Xchg(be, 1, self.nvars, self.ninterfpts)

    def xchg_items(self, field):
        """(peer, tag, host send, host receive) of a field's exchange."""
        x = self._xs if field == 'scal' else self._xv
        return x, (self.rhsrank, 0 if field == 'scal' else 1, x.hsend,
                   x.hrecv)


class EulerMPIInters(BaseMPIInters):
    def __init__(self, *args, **kwargs):
        super().__init__(*args, **kwargs)
        be = self._be
        rsolver = self.cfg.get('solver-interfaces', 'riemann-solver')
        p_min = riemann_p_min(self.cfg, be)
        self._tplargs = dict(ndims=self.ndims, nvars=self.nvars,
                             rsolver=rsolver, c=self.c, p_min=p_min)
        be.pointwise.register('pyfr.solvers.euler.kernels.mpicflux')
        self.kernels['scal_pack'] = lambda: be.kernel(
            'pack_view', self.scal_lhs, self._xs.send)
        self.kernels['comm_flux'] = lambda: be.kernel(
            'mpicflux', tplargs=self._tplargs, dims=[self.ninterfpts],
            ul=self.scal_lhs, ur=self._xs.rview, nl=self._pnorm_lhs)


class NavierStokesMPIInters(BaseMPIInters):
    def __init__(self, be, lhs, rhsrank, elemap, cfg, rank):
        super().__init__(be, lhs, rhsrank, elemap, cfg, rank)
        self._vect_lhs = self._vect_view(lhs, 'get_vect_fpts_for_inters')
        self._comm_lhs = self._scal_view(lhs, 'get_comm_fpts_for_inters')
        self._xv = _Xchg(be, self.ndims, self.nvars, self.ninterfpts)
        self.c |= cfg.items_as('solver-interfaces', float)

        # cflux(l, r, n_l) = -cflux(r, l, n_r) and conu(l, r) = conu(r, l)
        # need one of the two partitions to take -beta; which one follows
        # from the two ranks as in pyfr/solvers/baseadvecdiff/
        # inters.py:47-56
        if (rank + rhsrank) % 2:
            self.c['ldg-beta'] *= 1.0 if rank > rhsrank else -1.0
        else:
            self.c['ldg-beta'] *= 1.0 if rhsrank > rank else -1.0

        rsolver = cfg.get('solver-interfaces', 'riemann-solver')
        visc_corr = cfg.get('solver', 'viscosity-correction', 'none')
        self._tplargs = dict(ndims=self.ndims, nvars=self.nvars,
                             rsolver=rsolver, visc_corr=visc_corr,
                             shock_capturing='none', c=self.c,
                             p_min=riemann_p_min(cfg, be))
        be.pointwise.register('pyfr.solvers.navstokes.kernels.mpiconu')
        be.pointwise.register('pyfr.solvers.navstokes.kernels.mpicflux')
        self.kernels['scal_pack'] = lambda: be.kernel(
            'pack_view', self.scal_lhs, self._xs.send)
        self.kernels['vect_pack'] = lambda: be.kernel(
            'pack_view', self._vect_lhs, self._xv.send)
        self.kernels['con_u'] = lambda: be.kernel(
            'mpiconu', tplargs=self._tplargs, dims=[self.ninterfpts],
            ulin=self.scal_lhs, urin=self._xs.rview, ulout=self._comm_lhs,
            urout=self._xs.jview)
        self.kernels['comm_flux'] = lambda: be.kernel(
            'mpicflux', tplargs=self._tplargs, dims=[self.ninterfpts],
            ul=self.scal_lhs, ur=self._xs.rview, gradul=self._vect_lhs,
            gradur=self._xv.rview, nl=self._pnorm_lhs)


# ---------------------------------------------------------------------------
# Boundary conditions (pyfr/solvers/baseadvec/inters.py:74-116,
# pyfr/solvers/euler/inters.py:53-112, pyfr/solvers/navstokes/inters.py:66-150)
# ---------------------------------------------------------------------------

# The constants each boundary type reads from its [soln-bcs-<name>] section
BC_OPTS = {
    'sup-in-fa': ['rho', 'p', 'u', 'v', 'w'],
    'char-riem-inv': ['rho', 'p', 'u', 'v', 'w'],
    'no-slp-isot-wall': ['u', 'v', 'w'],
    'sub-in-frv': ['rho', 'u', 'v', 'w'],
    'sub-out-fp': ['p'],
    'sub-in-ftpttang': [],
    'sup-out-fn': [], 'slp-adia-wall': [], 'no-slp-adia-wall': [],
    # (the pressure comes from the controller, pyfr_gb300/solvers/
    # bccontrol.py)
    'char-riem-inv-mass-flow': ['rho', 'u', 'v', 'w'],
    'char-riem-inv-pressure': ['rho', 'u', 'v', 'w'],
}
# Velocity components that default to zero
_ZERO_UVW = {'no-slp-isot-wall', 'sub-in-frv'}
EULER_BCS = {'sup-in-fa', 'sup-out-fn', 'slp-adia-wall', 'char-riem-inv',
             'char-riem-inv-mass-flow', 'char-riem-inv-pressure'}
CONTROLLED_BCS = {'char-riem-inv-mass-flow': 'mass-flow',
                  'char-riem-inv-pressure': 'pressure'}


class BaseBCInters(BaseIntInters):
    """One boundary: its faces (the left side only), the view of the
    flux-point field over them, scaled normals, and the boundary type with
    its constants from ``[soln-bcs-<name>]``."""

    def __init__(self, be, lhs, elemap, cfgsect, cfg):
        from pyfr_gb300.backend.lib import BC, BC_TYPES
        from pyfr_gb300.solvers.elements import npeval

        self._be = be
        self.elemap = elemap
        self.cfg = cfg
        self.lhs, self.rhs = lhs, None
        self.cfgsect = cfgsect
        self.name = cfgsect.removeprefix('soln-bcs-')

        first = next(iter(elemap.values()))
        self.ndims, self.nvars = first.ndims, first.nvars
        self.ninters = len(lhs)
        self.ninterfpts = sum(elemap[et].nfacefpts[fi]*len(ei)
                              for et, fi, ei in lhs.items())
        self.c = cfg.items_as('constants', float)
        self.kernels = {}

        self.type = cfg.get(cfgsect, 'type')
        if self.type not in self.bctypes:
            raise NotImplementedError(f'Boundary type {self.type!r} is not '
                                      'provided')

        # Values: expressions of position and time, with [constants]
        # substituted (pyfr/solvers/baseadvec/inters.py:81-116); constant
        # ones are folded to numbers
        from pyfr_gb300.bcexpr import BCExpr
        vals, self.exprs = {}, {}
        opts = [k for k in BC_OPTS[self.type]
                if not (k in 'uvw' and 'uvw'.index(k) >= self.ndims)]
        if self.type == 'no-slp-isot-wall':
            opts.append('cpTw')
        for k in opts:
            default = '0' if self.type in _ZERO_UVW and k in 'uvw' else None
            expr = cfg.getexpr(cfgsect, k, default)
            if expr is None:
                raise ValueError(f'{cfgsect}: {k} is required')
            ex = BCExpr(str(expr), self.ndims)
            if ex.const is not None:
                vals[k] = ex.const
            else:
                vals[k] = 0.0
                self.exprs[k] = ex

        def ev(k):
            return float(npeval(cfg.get(cfgsect, k), dict(self.c)))

        vc = []
        if self.type == 'no-slp-isot-wall':
            pass
        elif self.type == 'sub-in-ftpttang':
            # Total state and inflow direction
            # (pyfr/solvers/navstokes/inters.py:169-193)
            vals['cpTt'], vals['pt'] = ev('cpTt'), ev('pt')
            theta = ev('theta')*np.pi/180
            vc = [np.cos(theta), np.sin(theta), 1.0]
            if self.ndims == 3:
                phi = ev('phi')*np.pi/180
                vc = [vc[0]*np.sin(phi), vc[1]*np.sin(phi), np.cos(phi)]
            vc = vc[:self.ndims]
        self.bcvals = vals
        self.bc = BC(type=BC_TYPES[self.type], rho=vals.get('rho', 0.0),
                     p=vals.get('p', 0.0), cpTw=vals.get('cpTw', 0.0),
                     cpTt=vals.get('cpTt', 0.0), pt=vals.get('pt', 0.0))
        for i, k in enumerate('uvw'[:self.ndims]):
            self.bc.u[i] = vals.get(k, 0.0)
        for i, v in enumerate(vc):
            self.bc.vc[i] = v

        # Memory order of the one side (pyfr/solvers/baseadvec/inters.py:90)
        scal = {t: e._scal_fpts for t, e in elemap.items()}
        self._perm = self._perm_for_field(lhs, scal)
        self._pnorm_lhs = self._const_mat(lhs, 'get_pnorms_for_inters')

        # The controller of a controlled characteristic boundary, whose
        # pressure p(t) = ic + im*t the kernels form with the stage time
        self.controller = None
        if self.type in CONTROLLED_BCS:
            from pyfr_gb300.solvers.bccontrol import ControlledBC
            self.controller = ControlledBC(be, cfg, cfgsect, elemap, lhs,
                                           CONTROLLED_BCS[self.type],
                                           first.con_to_pri)

        # Programs of the expression values and the point coordinates
        self.time_dependent = any(e.uses_t for e in self.exprs.values()) \
            or self.controller is not None
        self._prog = self._ploc = None
        if self.exprs:
            from pyfr_gb300.backend.lib import BCOp
            from pyfr_gb300.bcexpr import pack
            names = ['rho', 'p', 'u', 'v', 'w', 'cpTw']
            arr, spans = pack([self.exprs[k].prog if k in self.exprs else []
                               for k in names])
            for f, (start, n) in enumerate(spans):
                self.bc.expr_start[f], self.bc.expr_len[f] = start, n
            assert arr.itemsize == C.sizeof(BCOp)
            self._prog = be.const_matrix(arr.view(np.int64)[None, :],
                                         dtype=np.int64)
            self._ploc = self._const_mat(lhs, 'get_ploc_for_inters')

    def bind_device(self, tmat):
        """Point the boundary values at their programs, coordinates and
        the stage time (element 1 of ``tmat``), once memory is committed."""
        if self.exprs:
            self.bc.prog = self._prog.data
            self.bc.ploc = self._ploc.data
            self.bc.ldp = self._ploc.leaddim
        if self.exprs or self.controller:
            self.bc.t_dev = tmat.data + 8
        if self.controller:
            self.bc.ctrl = self.controller.ctrl.data

    def values_at(self, t):
        """Host values of the options at every boundary point at time t,
        in the kernels' point order (for checking)."""
        out = dict(self.bcvals)
        if self.exprs:
            x = inter_arrays(self.lhs, 'get_ploc_for_inters', self.elemap,
                             self._perm)[0].T
            for k, ex in self.exprs.items():
                out[k] = ex.eval_np(x, t)
        return out


class EulerBCInters(BaseBCInters):
    bctypes = EULER_BCS

    def __init__(self, *args, **kwargs):
        super().__init__(*args, **kwargs)
        rsolver = self.cfg.get('solver-interfaces', 'riemann-solver')
        self._tplargs = dict(ndims=self.ndims, nvars=self.nvars,
                             rsolver=rsolver, c=self.c, bctype=self.type,
                             bc=self.bc, p_min=riemann_p_min(self.cfg,
                                                             self._be))
        self._be.pointwise.register('pyfr.solvers.euler.kernels.bccflux')
        self.kernels['comm_flux'] = lambda: self._be.kernel(
            'bccflux', tplargs=self._tplargs, dims=[self.ninterfpts],
            ul=self.scal_lhs, nl=self._pnorm_lhs)


class NavierStokesBCInters(BaseBCInters):
    bctypes = set(BC_OPTS)

    def __init__(self, *args, **kwargs):
        super().__init__(*args, **kwargs)
        be, cfg = self._be, self.cfg
        self._vect_lhs = self._vect_view(self.lhs, 'get_vect_fpts_for_inters')
        self._comm_lhs = self._scal_view(self.lhs, 'get_comm_fpts_for_inters')
        self.c |= cfg.items_as('solver-interfaces', float)

        rsolver = cfg.get('solver-interfaces', 'riemann-solver')
        visc_corr = cfg.get('solver', 'viscosity-correction', 'none')
        self._tplargs = dict(ndims=self.ndims, nvars=self.nvars,
                             rsolver=rsolver, visc_corr=visc_corr,
                             shock_capturing=cfg.get('solver',
                                                     'shock-capturing',
                                                     'none'),
                             c=self.c, bctype=self.type, bc=self.bc,
                             p_min=riemann_p_min(cfg, be))
        self.artvisc = None
        be.pointwise.register('pyfr.solvers.navstokes.kernels.bcconu')
        be.pointwise.register('pyfr.solvers.navstokes.kernels.bccflux')
        self.kernels['con_u'] = lambda: be.kernel(
            'bcconu', tplargs=self._tplargs, dims=[self.ninterfpts],
            ulin=self.scal_lhs, ulout=self._comm_lhs, nlin=self._pnorm_lhs)
        self.kernels['comm_flux'] = lambda: be.kernel(
            'bccflux', tplargs=self._tplargs, dims=[self.ninterfpts],
            ul=self.scal_lhs, gradul=self._vect_lhs, nl=self._pnorm_lhs,
            **({'artvisc': self.artvisc} if self.artvisc is not None else {}))
