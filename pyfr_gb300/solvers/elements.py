"""Element types of the Euler and Navier-Stokes systems.

Each class allocates its scratch fields on the backend and declares its
kernels exactly as the reference elements do: same kernel names, same
operator expressions, same arguments
(``pyfr/solvers/base/elements.py:218-266``,
``pyfr/solvers/baseadvec/elements.py:61-128``,
``pyfr/solvers/baseadvecdiff/elements.py:26-120``,
``pyfr/solvers/euler/elements.py:149-206``,
``pyfr/solvers/navstokes/elements.py:30-128``).

Geometry is that of linear (multilinear) elements: the metric terms are
computed from the vertices; the kernels either recompute them at each
solution point from the vertices ('linear' kernel type, as the reference
does for uncurved elements) or read them from stored per-point arrays
('curved' kernel type).
"""

from functools import cached_property

import numpy as np

from pyfr_gb300.backend.types import NullKernel
from pyfr_gb300.mesh import fuzzy_face_order
from pyfr_gb300.shapes import SHAPES, adjugate_det, get_shape


# Point sets used when the configuration names none (the reference requires
# them in the configuration: solver-elements-<etype> soln-pts and
# solver-interfaces-<kind> flux-pts)
DEFAULT_UPTS = {'quad': 'gauss-legendre', 'hex': 'gauss-legendre',
                'tri': 'alpha-opt', 'tet': 'alpha-opt',
                'pri': 'alpha-opt~gauss-legendre-lobatto',
                'pyr': 'gauss-legendre'}
DEFAULT_FPTS = {'line': 'gauss-legendre', 'quad': 'gauss-legendre',
                'tri': 'alpha-opt'}


_NPEVAL_SYMS = {k: getattr(np, k) for k in
                ('sin', 'cos', 'tan', 'exp', 'log', 'sqrt', 'tanh', 'sinh',
                 'cosh', 'arctan2', 'abs', 'pi')}
_NPEVAL_SYMS |= {'pow': np.power, 'min': np.minimum, 'max': np.maximum,
                 'atan2': np.arctan2, 'fabs': np.abs}


def npeval(expr, env):
    """Evaluate an initial-condition expression over numpy arrays."""
    if '**' in expr or '^' in expr:
        raise ValueError('Direct exponentiation is not supported; use pow')
    return eval(expr, {'__builtins__': {}}, _NPEVAL_SYMS | env)


class BaseElements:
    # Set by the system: every flux point lies on an interior interface
    comm_covered = False
    # Set by the system: the device matrix whose element 1 is the stage time
    tmat = None
    src_uses_x = src_uses_u = src_uses_t = False
    def __init__(self, etype, eles, cfg):
        self.cfg = cfg
        self.eles = eles
        self.nspts, self.neles, self.ndims = eles.shape

        order = cfg.getint('solver', 'order')
        upts = cfg.get(f'solver-elements-{etype}', 'soln-pts',
                       DEFAULT_UPTS[etype])
        fpts = {k: cfg.get(f'solver-interfaces-{k}', 'flux-pts',
                           DEFAULT_FPTS[k])
                for k in {k for k, _, _ in SHAPES[etype].faces}}
        self.basis = get_shape(etype, order, upts, fpts)
        self.name = etype

        # Flux anti-aliasing (pyfr/solvers/baseadvec/elements.py:69-90):
        # the flux is evaluated at the points of a quadrature rule and
        # projected back; with 'surf-flux' the flux points are those of a
        # face quadrature rule (pyfr/shapes.py:147-227)
        aa = {a.strip() for a in cfg.get('solver', 'anti-alias',
                                         'none').split(',')} - {'none'}
        if aa - {'flux', 'surf-flux'}:
            raise ValueError('Invalid anti-alias options')
        if 'surf-flux' in aa and order > 0:
            self.basis.set_surf_rules(self._surf_rules(cfg, order))
        self.antialias = 'flux' in aa and order > 0
        if self.antialias:
            rule = cfg.get(f'solver-elements-{etype}', 'quad-pts', None)
            if rule is not None:
                from pyfr_gb300.quadrules import parse_rule
                pts, wts = parse_rule(rule, self.ndims)
                if wts is None:
                    raise ValueError('quad-pts needs quadrature weights')
                self.basis.set_qrule(pts, wts)

        self.convars = self.convarnames(self.ndims)
        self.nvars = len(self.convars)
        self._srctplargs = self._source_tplargs(cfg)
        self.nupts = self.basis.nupts
        self.nfpts = self.basis.nfpts
        self.nfacefpts = self.basis.nfacefpts
        self.kernels = {}
        self._be = None

    def _source_tplargs(self, cfg):
        """Template arguments of the source plugin's macro
        (pyfr/plugins/source.py:15-31): one expression per conserved
        variable of x, y, z (as ploc[i]), the conserved variables (as u[i])
        and t, with [constants] substituted; None without the plugin."""
        sect = 'solver-plugin-source'
        if not cfg.hassect(sect):
            return None
        from pyfr_gb300.bcexpr import BCExpr
        subs = dict(x='ploc[0]', y='ploc[1]', z='ploc[2]', abs='fabs',
                    pi=repr(np.pi))
        subs |= {v: f'u[{i}]' for i, v in enumerate(self.convars)}
        exprs = [cfg.getexpr(sect, v, subs=subs) for v in self.convars]
        parsed = [BCExpr(e, self.ndims, self.nvars) for e in exprs]
        self.src_uses_x = any(p.uses_x for p in parsed)
        self.src_uses_u = any(p.uses_u for p in parsed)
        self.src_uses_t = any(p.uses_t for p in parsed)
        return dict(ndims=self.ndims, nvars=self.nvars,
                    src_macros=[('pyfr.plugins.kernels.source', 'source')],
                    src_exprs=exprs)

    @property
    def has_src_macros(self):
        return self._srctplargs is not None

    def _surf_rules(self, cfg, order):
        """The face quadrature rule of each face kind for surface-flux
        anti-aliasing: ``[solver-interfaces-<kind>] quad-pts`` given
        literally, or Gauss-Legendre with ``quad-npts`` points (a square
        number on quadrilaterals), by default (p + 2) points per
        direction, the reference's default rules for lines and
        quadrilaterals."""
        from pyfr_gb300.quadrules import parse_rule, tensor_rule
        rules = {}
        for kind in {k for k, _, _ in self.basis.faces}:
            sect = f'solver-interfaces-{kind}'
            nd = {'line': 1, 'quad': 2, 'tri': 2}[kind]
            if cfg.hasopt(sect, 'quad-pts'):
                pts, wts = parse_rule(cfg.get(sect, 'quad-pts'), nd)
                if wts is None:
                    raise ValueError('quad-pts needs quadrature weights')
            elif kind == 'tri':
                raise NotImplementedError('Surface anti-aliasing on '
                                          'triangular faces needs a '
                                          'literal quad-pts rule')
            else:
                n1 = order + 2
                if cfg.hasopt(sect, 'quad-npts'):
                    n = cfg.getint(sect, 'quad-npts')
                    n1 = round(n**(1/nd))
                    if n1**nd != n:
                        raise ValueError(f'{sect}: quad-npts {n} is not a '
                                         'tensor-product rule')
                elif cfg.hasopt(sect, 'quad-deg'):
                    raise NotImplementedError(f'{sect}: give quad-pts or '
                                              'quad-npts')
                pts, wts = tensor_rule('gauss-legendre', n1, nd)
            rules[kind] = (pts, wts)
        return rules

    # ---- geometry (linear elements) -----------------------------------------

    def ploc_at_np(self, pts):
        pts = getattr(self.basis, pts) if isinstance(pts, str) else pts
        sf = self.basis.shape_fn(pts)                    # (npts, nverts)
        # (as one matrix product: sf @ eles over the vertex index)
        nv, ne, nd = self.eles.shape
        ploc = (sf @ self.eles.reshape(nv, ne*nd)).reshape(-1, ne, nd)
        return ploc.transpose(0, 2, 1)                   # (npts, ndims, neles)

    def _jac_at(self, pts):
        pts = getattr(self.basis, pts) if isinstance(pts, str) else pts
        dsf = self.basis.shape_jac(pts)                  # (npts, i, nverts)
        npt, ni, nv = dsf.shape
        _, ne, nd = self.eles.shape
        J = dsf.reshape(npt*ni, nv) @ self.eles.reshape(nv, ne*nd)
        return J.reshape(npt, ni, ne, nd).transpose(0, 1, 3, 2)  # (p, i, j, e)

    def smats_djac_at_np(self, pts):
        """Adjugate metric S[i][j] (npts, ndims, ndims, neles) and |J|."""
        key = pts if isinstance(pts, str) else None
        cache = self.__dict__.setdefault('_smats_cache', {})
        if key in cache:
            return cache[key]
        s, d = adjugate_det(self._jac_at(pts))
        if key is not None:
            cache[key] = (s, d)
        return s, d

    def smat_at_np(self, pts):
        s, _ = self.smats_djac_at_np(pts)
        return s.transpose(1, 0, 2, 3)      # (ndims_i, npts, ndims_j, neles)

    def rcpdjac_at_np(self, pts):
        _, d = self.smats_djac_at_np(pts)
        if np.any(d < -1e-5):
            raise RuntimeError('Negative mesh Jacobians detected')
        return 1.0 / d

    @cached_property
    def _pnorm_fpts(self):
        s, _ = self.smats_djac_at_np('fpts')             # (p, l, k, e)
        pn = np.einsum('plke,pl->pek', s, self.basis.norm_fpts)
        if np.any(np.sqrt(np.einsum('...i,...i', pn, pn)) < 1e-10):
            raise RuntimeError('Zero face normals detected')
        return pn                                        # (nfpts, neles, ndims)

    @cached_property
    def plocfpts(self):
        return self.ploc_at_np('fpts').transpose(0, 2, 1)   # (nfpts, neles, d)

    @cached_property
    def srtd_face_fpts(self):
        """Flux-point indices of each face, in physical-coordinate order,
        per element: list over faces of (neles, nfacefpts) arrays."""
        out = []
        for ffpts in self.basis.facefpts:
            ffpts = np.asarray(ffpts)
            coords = self.plocfpts[ffpts].transpose(1, 2, 0)
            out.append(ffpts[fuzzy_face_order(coords)])
        return out

    # ---- initial conditions ------------------------------------------------

    def set_ics_from_cfg(self):
        consts = self.cfg.items_as('constants', float)
        coords = self.ploc_at_np('upts')                 # (nupts, ndims, neles)
        env = consts | dict(zip('xyz', coords.swapaxes(0, 1)))
        pris = [np.broadcast_to(npeval(self.cfg.getexpr('soln-ics', v), env),
                                (self.nupts, self.neles))
                for v in self.privarnames(self.ndims)]

        ics = np.empty((self.nupts, self.nvars, self.neles))
        for i, v in enumerate(self.pri_to_con(pris, self.cfg)):
            ics[:, i] = v
        return ics

    # ---- backend set-up -------------------------------------------------------

    @property
    def mesh_regions(self):
        off = self.linoff
        if off == 0:
            return {'linear': self.neles}
        elif off >= self.neles:
            return {'curved': self.neles}
        return {'curved': off, 'linear': self.neles - off}

    def _slice_mat(self, mat, region):
        if mat is None:
            return None
        off = self.linoff
        if len(mat.ioshape) >= 3:
            off *= mat.ioshape[-2]
        else:
            off = min(off, mat.ncol)
        if region == 'curved':
            return mat.slice(None, None, 0, off)
        return mat.slice(None, None, off, mat.ncol)

    def _make_sliced_kernel(self, kseq):
        kl = list(kseq)
        if len(kl) > 1:
            return self._be.unordered_meta_kernel(kl, [self.linoff])
        return kl[0]

    def set_backend(self, backend, nonce, linoff):
        self._be = be = backend
        self._nonce = nonce
        self.grad_fusion = not be.blocks

        csub = backend.csubsz
        self.linoff = linoff - linoff % -csub if self.basis.order >= 2 else self.neles

        ndims, nvars, neles = self.ndims, self.nvars, self.neles
        abufs = []

        def alloc(ex, shape):
            m = be.matrix(shape, extent=nonce + ex, tags={'align'})
            abufs.append(m)
            return m

        sbufs = self._scratch_bufs
        if 'scal_fpts' in sbufs:
            self._scal_fpts = alloc('scal_fpts', (self.nfpts, nvars, neles))
        # (with flux anti-aliasing the Euler flux lives at the quadrature
        # points instead)
        if 'vect_upts' in sbufs and not (self.antialias and
                                         'grad_upts' not in sbufs):
            self._vect_upts = alloc('vect_upts', (ndims, self.nupts, nvars, neles))
        if 'vect_fpts' in sbufs:
            self._vect_fpts = alloc('vect_fpts', (ndims, self.nfpts, nvars, neles))
        if 'grad_upts' in sbufs:
            self._grad_upts = alloc('grad_upts', (ndims, self.nupts, nvars, neles))
        elif hasattr(self, '_vect_upts'):
            self._grad_upts = self._vect_upts
        if 'vect_fpts' in sbufs:
            self._comm_fpts = self._vect_fpts.slice(0, self.nfpts)

        self.scal_upts = []

    def alloc_bank(self, extent, ic=None):
        m = self._be.matrix((self.nupts, self.nvars, self.neles), ic,
                            extent=extent, tags={'align'})
        self.scal_upts.append(m)
        return m

    def opmat(self, expr):
        key = ('opmat', expr)
        if key not in self.__dict__:
            self.__dict__[key] = self._be.const_matrix(
                self.basis.opmat(expr), tags={expr, 'align'})
        return self.__dict__[key]

    def release_host_geometry(self):
        """Drop cached host-side metric arrays (recomputed if needed)."""
        for k in ('_smats_cache', '_pnorm_fpts', 'plocfpts'):
            self.__dict__.pop(k, None)

    def _cached(self, key, fn):
        if key not in self.__dict__:
            self.__dict__[key] = fn()
        return self.__dict__[key]

    def rcpdjac_at(self, name, side=None):
        m = self._cached(('rcpdjac', name), lambda: self._be.const_matrix(
            self.rcpdjac_at_np(name), tags={'align'}))
        return self._slice_mat(m, side) if side else m

    def curved_smat_at(self, name):
        return self._cached(('csmat', name), lambda: self._be.const_matrix(
            self.smat_at_np(name)[..., :self.linoff], tags={'align'}))

    def ploc_at(self, name, side=None):
        m = self._cached(('ploc', name), lambda: self._be.const_matrix(
            self.ploc_at_np(name), tags={'align'}))
        return self._slice_mat(m, side) if side else m

    @cached_property
    def upts(self):
        return self._be.const_matrix(self.basis.upts)

    @cached_property
    def qpts(self):
        return self._be.const_matrix(self.basis.qpts)

    # ---- interface helpers (pyfr/solvers/base/elements.py:446-469) --------

    def get_ploc_for_inters(self, eidxs, fidx):
        """Physical coordinates of the face's flux points in their sorted
        order (pyfr/solvers/base/elements.py, get_ploc_for_inters)."""
        if not hasattr(self, '_ploc_fpts_np'):
            self._ploc_fpts_np = self.ploc_at_np('fpts')  # (nfpts, nd, ne)
        fpts_idx = self.srtd_face_fpts[fidx][eidxs]
        pl = self._ploc_fpts_np[fpts_idx, :, eidxs[:, None]]
        return pl.reshape(-1, self.ndims),

    def get_pnorms_for_inters(self, eidxs, fidx):
        fpts_idx = self.srtd_face_fpts[fidx][eidxs]
        pn = self._pnorm_fpts[fpts_idx, eidxs[:, None]]
        return pn.reshape(-1, self.ndims),

    def _inters_map(self, eidxs, fidx, mid, rmap, lda=None):
        nfp = self.nfacefpts[fidx]
        n = len(eidxs)
        cmap = np.repeat(eidxs, nfp)
        if lda is None:
            return np.full(n*nfp, mid), rmap.ravel(), cmap
        return np.full(n*nfp, mid), rmap.ravel(), cmap, np.full(n*nfp, lda)

    def get_vect_fpts_for_inters(self, eidxs, fidx):
        rmap = self.srtd_face_fpts[fidx][eidxs]
        return self._inters_map(eidxs, fidx, self._vect_fpts.mid, rmap,
                                self.nfpts)

    def get_comm_fpts_for_inters(self, eidxs, fidx):
        rmap = self.srtd_face_fpts[fidx][eidxs]
        return self._inters_map(eidxs, fidx, self._comm_fpts.mid, rmap)


class FluidElements:
    """Variables and conversions of the compressible equations
    (``pyfr/solvers/euler/elements.py:71-136``)."""

    @staticmethod
    def privarnames(ndims):
        return ['rho', 'u', 'v', 'p'] if ndims == 2 else \
               ['rho', 'u', 'v', 'w', 'p']

    @staticmethod
    def convarnames(ndims):
        return ['rho', 'rhou', 'rhov', 'E'] if ndims == 2 else \
               ['rho', 'rhou', 'rhov', 'rhow', 'E']

    @staticmethod
    def pri_to_con(pris, cfg):
        rho, p = pris[0], pris[-1]
        rhovs = [rho*c for c in pris[1:-1]]
        gamma = cfg.getfloat('constants', 'gamma')
        E = p/(gamma - 1) + 0.5*rho*sum(c*c for c in pris[1:-1])
        return [rho, *rhovs, E]

    @staticmethod
    def con_to_pri(cons, cfg):
        rho, E = cons[0], cons[-1]
        vs = [rhov/rho for rhov in cons[1:-1]]
        gamma = cfg.getfloat('constants', 'gamma')
        p = (gamma - 1)*(E - 0.5*rho*sum(v*v for v in vs))
        return [rho, *vs, p]


class _WavespeedMixin:
    def init_wavespeed(self):
        """Per-element wave speed for the CFL controller
        (pyfr/solvers/euler/elements.py:21-66)."""
        be = self._be
        be.pointwise.register('pyfr.solvers.euler.kernels.wavespeed')
        self._wspd = be.matrix((1, self.neles), tags={'align'})
        self.kernels['wavespeed'] = lambda uin: self._wavespeed_kernel(uin)
        return self._wspd

    def _wavespeed_kernel(self, uin):
        be, r, s = self._be, self.mesh_regions, self._slice_mat
        tplargs = dict(ndims=self.ndims, nvars=self.nvars,
                       nverts=len(self.basis.linspts),
                       c=self.cfg.items_as('constants', float))
        kerns = []
        for rgn in ('curved', 'linear'):
            if rgn not in r:
                continue
            if rgn == 'curved':
                kw = dict(smats=self.curved_smat_at('upts'),
                          rcpdjac=self.rcpdjac_at('upts', 'curved'))
            else:
                kw = dict(verts=self.ploc_at('linspts', 'linear'),
                          upts=self.upts)
            # (each region writes its own elements' entries)
            kerns.append(be.kernel(
                'wavespeed', tplargs=tplargs | {'ktype': rgn},
                dims=[self.nupts, r[rgn]], u=s(self.scal_upts[uin], rgn),
                wspd=s(self._wspd, rgn), **kw))
        return self._make_sliced_kernel(kerns)

    def dt_cfl(self):
        """Largest stable step of each element: 1/((2p + 1) wspd)."""
        with np.errstate(divide='ignore'):
            w = (2*self.basis.order + 1)*self._wspd.get()[0]
            return np.nan_to_num(1/w, posinf=0.0)


class _DivergenceMixin:
    def _divergence_kernels(self):
        """tdivtpcorf, tdivtconf and negdivconf
        (pyfr/solvers/baseadvec/elements.py:91-120), or, with fused
        operators, all three as one kernel:
        R = -(1/|J|)((M1 - M3.M2) F + M3 Fc)."""
        be, kernels = self._be, self.kernels
        src = self._source_kernels()
        # (with flux anti-aliasing the flux lives at the quadrature points
        # and is projected back by M9)
        m132, vect = ('(M1 - M3*M2)*M9', self._vect_qpts) if \
            getattr(self, 'antialias', False) else \
            ('M1 - M3*M2', self._vect_upts)
        if be.fuse_operators:
            kernels['tdivtconf_cat'] = lambda fout: be.kernel(
                'mul_cat', self.opmat(m132), vect,
                self.opmat('M3'), self._scal_fpts, out=self.scal_upts[fout],
                alpha=-1.0, rowscale=self.rcpdjac_at('upts'))
            # (then the source terms, added to -(1/|J|) div F)
            if src:
                kernels['addsrc'] = lambda fout: be.kernel(
                    'addsrc', tplargs=self._srctplargs,
                    dims=[self.nupts, self.neles], r=self.scal_upts[fout],
                    **src())
            return

        kernels['tdivtpcorf'] = lambda fout: be.kernel(
            'mul', self.opmat(m132), vect, out=self.scal_upts[fout])
        kernels['tdivtconf'] = lambda fout: be.kernel(
            'mul', self.opmat('M3'), self._scal_fpts,
            out=self.scal_upts[fout], beta=1.0)
        kernels['negdivconf'] = lambda fout: be.kernel(
            'negdivconf', tplargs=self._srctplargs or dict(
                ndims=self.ndims, nvars=self.nvars, src_macros=[]),
            dims=[self.nupts, self.neles], tdivtconf=self.scal_upts[fout],
            rcpdjac=self.rcpdjac_at('upts'), **(src() if src else {}))

    def _source_kernels(self):
        """With source terms: the copy of the solution they read (the
        right-hand side may overwrite its input bank) and evalsrcmacros
        (pyfr/solvers/baseadvec/elements.py:100-126); returns a function
        giving the source arguments of negdivconf, or None."""
        if self._srctplargs is None:
            return None
        be, kernels = self._be, self.kernels
        be.pointwise.register('pyfr.solvers.baseadvec.kernels.evalsrcmacros')
        be.pointwise.register('pyfr_gb300.kernels.addsrc')
        if self.src_uses_u:
            self._scal_upts_cpy = be.matrix(
                (self.nupts, self.nvars, self.neles), tags={'align'})
            kernels['copy_soln'] = lambda uin: be.kernel(
                'copy', self._scal_upts_cpy, self.scal_upts[uin])

        def args():
            return dict(
                ploc=self.ploc_at('upts') if self.src_uses_x else None,
                u=self._scal_upts_cpy if self.src_uses_u else None,
                tmat=self.tmat)

        kernels['evalsrcmacros'] = lambda uin: be.kernel(
            'evalsrcmacros', tplargs=self._srctplargs,
            dims=[self.nupts, self.neles], u=self.scal_upts[uin],
            ploc=self.ploc_at('upts') if self.src_uses_x else None,
            tmat=self.tmat)
        return args


class EulerElements(_WavespeedMixin, _DivergenceMixin, FluidElements,
                    BaseElements):
    _scratch_bufs = {'scal_fpts', 'vect_upts'}

    def set_backend(self, backend, nonce, linoff):
        super().set_backend(backend, nonce, linoff)
        be, kernels = self._be, self.kernels

        be.pointwise.register('pyfr.solvers.baseadvec.kernels.negdivconf')
        be.pointwise.register('pyfr.solvers.euler.kernels.tflux')

        # Interpolate the solution to the flux points
        kernels['disu'] = lambda uin: be.kernel(
            'mul', self.opmat('M0'), self.scal_upts[uin], out=self._scal_fpts)

        # Transformed flux, at the solution points or, with flux
        # anti-aliasing, at the quadrature points
        tplargs = dict(ndims=self.ndims, nvars=self.nvars,
                       nverts=len(self.basis.linspts),
                       c=self.cfg.items_as('constants', float))
        r, s = self.mesh_regions, self._slice_mat
        if self.antialias:
            nd, nq = self.ndims, self.basis.nqpts
            ex = be.matrix((nq, self.nvars, self.neles), tags={'align'},
                           extent=self._nonce + 'scal_qpts')
            self._scal_qpts = ex
            self._vect_qpts = be.matrix((nd, nq, self.nvars, self.neles),
                                        tags={'align'},
                                        extent=self._nonce + 'vect_qpts')
            kernels['qptsu'] = lambda uin: be.kernel(
                'mul', self.opmat('M7'), self.scal_upts[uin],
                out=self._scal_qpts)
            npts, where = nq, 'qpts'

            def uin_mat(uin):
                return self._scal_qpts
            fmat = self._vect_qpts
        else:
            npts, where = self.nupts, 'upts'

            def uin_mat(uin):
                return self.scal_upts[uin]
            fmat = self._vect_upts
        tdisf = []
        if 'curved' in r:
            tdisf.append(lambda uin: be.kernel(
                'tflux', tplargs=tplargs | {'ktype': 'curved'},
                dims=[npts, r['curved']], u=s(uin_mat(uin), 'curved'),
                f=s(fmat, 'curved'), smats=self.curved_smat_at(where)))
        if 'linear' in r:
            tdisf.append(lambda uin: be.kernel(
                'tflux', tplargs=tplargs | {'ktype': 'linear'},
                dims=[npts, r['linear']], u=s(uin_mat(uin), 'linear'),
                f=s(fmat, 'linear'), verts=self.ploc_at('linspts', 'linear'),
                upts=getattr(self, where)))
        kernels['tdisf'] = lambda uin: self._make_sliced_kernel(
            k(uin) for k in tdisf)

        # Divergence of the partially corrected flux and the correction
        self._divergence_kernels()


class NavierStokesElements(_WavespeedMixin, _DivergenceMixin, FluidElements,
                           BaseElements):
    _scratch_bufs = {'scal_fpts', 'vect_fpts', 'vect_upts', 'grad_upts'}

    # Set by the system: the flux kernel stores the transformed gradient
    # (False: it leaves it in reference space, and the interface kernels
    # transform the face gradients with the affine elements' metrics)
    grad_writeback = True
    # Set by the system with the face metrics: this type's first column in
    # the interface kernels' metric matrix
    face_metric_col = 0

    def affine_metrics(self):
        """(S (ndims, ndims, neles) and 1/|J| (neles,)) of the elements
        when every one is linear and affine (the same metric terms at every
        point), else None."""
        from pyfr_gb300.backend.pointwise import affine, linear_metrics
        if self.linoff:
            return None
        sm, rj = linear_metrics(self.eles.transpose(0, 2, 1), self.basis.upts)
        if not affine(sm):
            return None
        return sm[:, 0], rj[0]

    def get_eidx_for_inters(self, eidxs, fidx):
        return np.repeat(eidxs + self.face_metric_col,
                         self.nfacefpts[fidx]).astype(np.int32),

    def set_backend(self, backend, nonce, linoff):
        super().set_backend(backend, nonce, linoff)
        be, kernels = self._be, self.kernels

        be.pointwise.register('pyfr.solvers.baseadvec.kernels.negdivconf')
        be.pointwise.register('pyfr.solvers.baseadvecdiff.kernels.gradcoru')
        be.pointwise.register('pyfr.solvers.navstokes.kernels.tflux')

        kernels['disu'] = lambda uin: be.kernel(
            'mul', self.opmat('M0'), self.scal_upts[uin], out=self._scal_fpts)

        # (not needed when the interfaces write the common solution to
        # both sides of every flux point: comm_covered, set by the system)
        if abs(self.cfg.getfloat('solver-interfaces', 'ldg-beta')) == 0.5:
            kernels['copy_fpts'] = lambda: NullKernel() \
                if self.comm_covered else be.kernel(
                    'copy', self._comm_fpts, self._scal_fpts)

        if be.fuse_operators:
            # Corrected gradient in one operator apply: [M4-M6.M0 | M6]
            # on the solution stacked over the common solution
            kernels['tgradcoru_upts_cat'] = lambda uin: be.kernel(
                'mul_cat', self.opmat('M4 - M6*M0'), self.scal_upts[uin],
                self.opmat('M6'), self._comm_fpts, out=self._grad_upts)
        else:
            kernels['tgradpcoru_upts'] = lambda uin: be.kernel(
                'mul', self.opmat('M4 - M6*M0'), self.scal_upts[uin],
                out=self._grad_upts)
            kernels['tgradcoru_upts'] = lambda: be.kernel(
                'mul', self.opmat('M6'), self._comm_fpts,
                out=self._grad_upts, beta=1.0)

        r, s = self.mesh_regions, self._slice_mat
        if self.antialias:
            # Flux anti-aliasing: the solution and the physical gradient
            # interpolated to the quadrature points, where the unfused flux
            # kernel runs (pyfr/solvers/baseadvecdiff/elements.py:103-116,
            # pyfr/solvers/navstokes/elements.py:60-123)
            nd, nq = self.ndims, self.basis.nqpts
            self._scal_qpts = be.matrix((nq, self.nvars, self.neles),
                                        tags={'align'},
                                        extent=self._nonce + 'scal_qpts')
            self._vect_qpts = be.matrix((nd, nq, self.nvars, self.neles),
                                        tags={'align'},
                                        extent=self._nonce + 'vect_qpts')
            kernels['qptsu'] = lambda uin: be.kernel(
                'mul', self.opmat('M7'), self.scal_upts[uin],
                out=self._scal_qpts)

            def gradcoru_qpts():
                nupts, vu, vq = self.nupts, self._grad_upts, self._vect_qpts
                if be.fuse_operators:
                    return be.kernel('mul_batched', self.opmat('M7'), vu, vq,
                                     nbatch=self.ndims)
                return be.unordered_meta_kernel([
                    be.kernel('mul', self.opmat('M7'),
                              vu.slice(i*nupts, (i + 1)*nupts),
                              vq.slice(i*nq, (i + 1)*nq))
                    for i in range(self.ndims)])
            kernels['gradcoru_qpts'] = gradcoru_qpts

        gtpl = dict(ndims=self.ndims, nvars=self.nvars,
                    nverts=len(self.basis.linspts))
        gradcoru_u = []
        if 'curved' in r:
            gradcoru_u.append(lambda: be.kernel(
                'gradcoru', tplargs=gtpl | {'ktype': 'curved'},
                dims=[self.nupts, r['curved']],
                gradu=s(self._grad_upts, 'curved'),
                smats=self.curved_smat_at('upts'),
                rcpdjac=self.rcpdjac_at('upts', 'curved')))
        if 'linear' in r:
            gradcoru_u.append(lambda: be.kernel(
                'gradcoru', tplargs=gtpl | {'ktype': 'linear'},
                dims=[self.nupts, r['linear']],
                gradu=s(self._grad_upts, 'linear'), upts=self.upts,
                verts=self.ploc_at('linspts', 'linear')))
        kernels['gradcoru_u'] = lambda: self._make_sliced_kernel(
            k() for k in gradcoru_u)

        def gradcoru_fpts():
            nupts, nfpts = self.nupts, self.nfpts
            vupts, vfpts = self._grad_upts, self._vect_fpts
            if be.fuse_operators:
                # The ndims products as one launch over ndims slices
                return be.kernel('mul_batched', self.opmat('M0'), vupts,
                                 vfpts, nbatch=self.ndims)
            muls = [be.kernel('mul', self.opmat('M0'),
                              vupts.slice(i*nupts, (i + 1)*nupts),
                              vfpts.slice(i*nfpts, (i + 1)*nfpts))
                    for i in range(self.ndims)]
            return be.unordered_meta_kernel(muls)
        kernels['gradcoru_fpts'] = gradcoru_fpts

        visc_corr = self.cfg.get('solver', 'viscosity-correction', 'none')
        sc = self.cfg.get('solver', 'shock-capturing', 'none')
        tplargs = dict(ndims=self.ndims, nvars=self.nvars,
                       nverts=len(self.basis.linspts),
                       c=self.cfg.items_as('constants', float),
                       shock_capturing=sc, visc_corr=visc_corr)
        aa = self.antialias
        pts = 'qpts' if aa else 'upts'
        npts = self.basis.nqpts if aa else self.nupts
        tdisf = []
        for rgn in ('curved', 'linear'):
            if rgn not in r:
                continue
            kw = dict(upts=getattr(self, pts))
            if rgn == 'curved':
                kw |= dict(smats=self.curved_smat_at(pts))
                if not aa:
                    kw |= dict(rcpdjac=self.rcpdjac_at('upts', 'curved'))
            else:
                kw |= dict(verts=self.ploc_at('linspts', 'linear'))
            if aa:
                kw |= dict(f=s(self._vect_qpts, rgn))
                tdisf.append((rgn, r[rgn], rgn, kw))
            else:
                kw |= dict(f=s(self._vect_upts, rgn),
                           gradu=s(self._grad_upts, rgn))
                tdisf.append((f'{rgn}-fused', r[rgn], rgn, kw))

        # (artificial viscosity at the points of the flux: set by the system
        # before the kernels are made)
        def avkw(rgn):
            if sc != 'artificial-viscosity':
                return {}
            return dict(artvisc=s(self.artvisc_upts, rgn))

        if aa:
            kernels['tdisf'] = lambda: self._make_sliced_kernel(
                be.kernel('tflux', tplargs=tplargs | {'ktype': kt},
                          dims=[npts, n], u=s(self._scal_qpts, rgn), **kw,
                          **avkw(rgn))
                for kt, n, rgn, kw in tdisf)
        else:
            kernels['tdisf_fused'] = lambda uin: self._make_sliced_kernel(
                be.kernel('tflux', tplargs=tplargs | {'ktype': kt},
                          dims=[npts, n], u=s(self.scal_upts[uin], rgn),
                          **kw, **avkw(rgn),
                          **({} if self.grad_writeback else
                             {'gradwb': False}))
                for kt, n, rgn, kw in tdisf)

        self._divergence_kernels()
