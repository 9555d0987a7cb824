"""Pointwise kernel provider of the ``b200`` backend.

The reference renders a Mako template per kernel module and compiles it at
run time (``pyfr/backends/base/provider.py:173-206``).  Here every module
on the right-hand-side path maps to a hand-written CUDA kernel of the
pyfrb200 library; ``register(modpath)`` exposes the kernel that module
defines under its name, and calling it takes the same arguments as the
reference's generated kernel: ``name(tplargs, dims, extrns={}, **args)``.
Scalar arguments that are not supplied become runtime-bindable
(``rtnames``), as with ``pyfr/backends/base/provider.py:134-141``.
"""

import ctypes as C

import numpy as np

from pyfr_gb300.shapes import ETYPE_OF, adjugate_det, linear_shape_jac

from pyfr_gb300.backend.lib import Gas
from pyfr_gb300.backend.types import BindableKernel, Kernel, NullKernel

# The Riemann solvers of pyfr/solvers/euler/kernels/rsolvers/ by the index
# the C ABI takes
RSOLVERS = {'rusanov': 0, 'hllc': 1, 'hll': 2, 'roe': 3, 'roem': 4,
            'exact': 5}

# Star-pressure floor of the exact solver when the caller gives none
# (pyfr/solvers/euler/inters.py:21-22: five FP64 machine epsilons)
P_MIN_DEFAULT = 5*float(np.finfo(np.float64).eps)


def _rsolver(tplargs):
    try:
        return RSOLVERS[tplargs['rsolver']]
    except KeyError:
        raise ValueError(f'Unknown Riemann solver '
                         f'{tplargs.get("rsolver")!r}') from None


def _gas(c, visc_corr='none', ref_state=None, p_min=P_MIN_DEFAULT):
    g = Gas(gamma=c['gamma'], mu=c.get('mu', 0.0), pr=c.get('Pr', 1.0),
            cpTref=c.get('cpTref', 1.0), cpTs=c.get('cpTs', 1.0),
            sutherland=int(visc_corr == 'sutherland'), p_min=p_min)
    if ref_state is not None:
        g.shifted = 1
        g.rho_ref, g.p_ref = ref_state[:2]
        for i, v in enumerate(ref_state[2] if len(ref_state) > 2 else ()):
            g.v_ref[i] = v
    return g


def _mat(m):
    """(device pointer, leading dimension) of a matrix argument."""
    if m is None:
        return None, 0
    return m.data, m.leaddim


def linear_metrics(verts, upts):
    """Adjugate metric terms S[i][j] (ndims, nupts, ndims, neles) and 1/|J|
    (nupts, neles) of linear elements at reference points ``upts``; verts
    has io-shape (nverts, ndims, neles) in the reference's vertex order,
    which with ndims identifies the element type.  Same arithmetic as the
    kernels' in-place computation for multilinear elements
    (pyfr/solvers/baseadvec/kernels/smats.mako:3-25) and the Jacobian
    expressions of the other linear shapes (pyfr/shapes.py)."""
    nverts, nd, ne = verts.shape
    try:
        etype = ETYPE_OF[nd, nverts]
    except KeyError:
        raise ValueError(f'No linear element with {nverts} vertices in '
                         f'{nd} dimensions') from None
    x = np.asarray(upts, dtype=float)
    dN = linear_shape_jac(etype, x)                     # (npts, nd, nverts)
    # J[p, i, j, e] as one matrix product over the vertex index
    npt = len(x)
    J = (dN.reshape(npt*nd, nverts) @ verts.reshape(nverts, nd*ne))
    S, d = adjugate_det(J.reshape(npt, nd, nd, ne))
    return S.transpose(1, 0, 2, 3), 1.0/d


# Geometry modes of the element kernels (the C ABI's `linear` argument)
GEOM_STORED, GEOM_VERTICES, GEOM_PER_ELEMENT = 0, 1, 2


def affine(smats, rtol=1e-13):
    """Whether every element's metric terms S (ndims, npts, ndims, neles)
    are the same at all its points (to rounding): true of affine elements
    (parallelograms, parallelepipeds, simplices)."""
    dev = np.abs(smats - smats[:, :1]).max(axis=(0, 1, 2))
    return bool(np.all(dev <= rtol*np.abs(smats).max(axis=(0, 1, 2))))


def _host_of(m):
    """Host copy of a constant matrix or of a whole-width slice of one."""
    if hasattr(m, '_host'):
        return m._host
    p = getattr(m, 'parent', None)
    if p is not None and hasattr(p, '_host') and m.ca == 0 and \
            m.cb == p.ncol and m.ra == 0 and m.rb == p.nrow:
        return p._host
    return None


def _unit_normal_rows(nlh):
    """(ndims + 1, n) rows of the unit normals and magnitudes of the
    scaled normals nlh (ndims, n), formed as the reference's interface
    kernels form them (pyfr/solvers/euler/kernels/intcflux.mako:12-13):
    mag = sqrt(n.n), unit = (1/mag) n."""
    nlh = np.asarray(nlh, dtype=np.float64)
    mag = np.sqrt(np.sum(nlh*nlh, axis=0))
    return np.vstack([(1/mag)*nlh, mag[None]])


def _view(v):
    """(base pointer, map pointer, row-stride pointer) of a view."""
    return (v.basedata, v.mapping.data,
            v.rstrides.data if v.rstrides is not None else None)


class PointwiseKernelProvider:
    def __init__(self, backend):
        self.backend = backend
        self._registered = {}
        self._metrics = {}

    @property
    def _sfx(self):
        return 'f64' if self.backend.fpdtype == np.float64 else 'f32'

    def _fn(self, name):
        return getattr(self.backend.lib, f'{name}_{self._sfx}')

    @property
    def _ix64(self):
        return int(self.backend.ixdtype == np.int64)

    def register(self, mod):
        """Expose the kernel defined by reference module ``mod``."""
        name = mod.rsplit('.', 1)[-1]
        builder = _BUILDERS.get(mod)

        def kernel_meth(tplargs, dims, extrns={}, **kwargs):
            if builder is None:
                raise NotImplementedError(
                    f'Kernel {name!r} of {mod} is not provided by the b200 '
                    'backend')
            return builder(self, tplargs, dims, extrns, **kwargs)

        self._registered[name] = mod
        setattr(self, name, kernel_meth)

    # ---- element kernels ---------------------------------------------------

    def _geom(self, tplargs, smats=None, rcpdjac=None, verts=None, upts=None):
        linear = 'linear' in tplargs.get('ktype', 'curved')
        # The kernels rebuild metrics in place for multilinear elements
        # only; other linear shapes always read stored terms
        multilin = tplargs.get('nverts', 2**tplargs['ndims']) == \
            2**tplargs['ndims']
        if linear and (self.backend.precompute_metrics or not multilin):
            # FP64 arithmetic is scarce on this GPU while bandwidth is not:
            # read stored metric terms (10 values) instead of rebuilding the
            # Jacobian from the vertices (~200 flops); affine elements keep
            # one set per element
            m = self._stored_metrics(verts, upts)
            if m is not None:
                smats, rcpdjac, per_ele = m
                return (GEOM_PER_ELEMENT if per_ele else GEOM_STORED,
                        _mat(smats), _mat(rcpdjac), (None, 0), (None, 0))
        if linear:
            if not multilin:
                raise ValueError('Linear-element kernels of this shape need '
                                 'the host copies of its vertices')
            return GEOM_VERTICES, (None, 0), (None, 0), _mat(verts), \
                _mat(upts)
        return GEOM_STORED, _mat(smats), _mat(rcpdjac), (None, 0), (None, 0)

    def _normals(self, nl):
        """(pointer, leading dimension, stored-unit flag) of the normals
        of an interface kernel: the unit normals and magnitudes formed
        once on the host when nl has a host copy, else nl itself."""
        h = _host_of(nl)
        if h is None:
            np_, nlp = _mat(nl)
            return np_, nlp, 0, nl
        key = ('unit', id(h))
        if key not in self._metrics:
            m = self.backend.const_matrix(_unit_normal_rows(h),
                                          tags={'align'})
            self._metrics[key] = (m, h)
        m = self._metrics[key][0]
        return m.data, m.leaddim, 1, m

    def _stored_metrics(self, verts, upts):
        vh, uh = _host_of(verts), _host_of(upts)
        if vh is None or uh is None:
            return None
        key = (id(vh), id(uh))
        if key not in self._metrics:
            be = self.backend
            sm, rj = linear_metrics(vh, uh)
            per_ele = self.backend.per_element_metrics and affine(sm)
            if per_ele:
                sm, rj = sm[:, :1], rj[:1]
            self._metrics[key] = (be.const_matrix(sm, tags={'align'}),
                                  be.const_matrix(rj, tags={'align'}),
                                  per_ele, vh, uh)
        return self._metrics[key][:3]

    def _tflux_euler(self, tplargs, dims, extrns, u, f, smats=None,
                     verts=None, upts=None):
        nupts, neles = dims
        lin, (sp, sl), _, (vp, vl), (upp, upl) = self._geom(
            tplargs, smats=smats, verts=verts, upts=upts)
        fn, gamma = self._fn('tflux_euler'), tplargs['c']['gamma']
        up, ul = _mat(u)
        fp, fl = _mat(f)
        nd = tplargs['ndims']
        gas = None

        if self.backend.ref_state is not None:
            # Shifted inputs: the flux less the reference state's
            fn = self._fn('tflux_euler_shift')
            gas = _gas(tplargs['c'], 'none', self.backend.ref_state)

            def run(stream):
                fn(nd, nupts, neles, lin, C.byref(gas), up, ul, fp, fl, sp, sl,
                   vp, vl, upp, upl, stream)
        else:
            def run(stream):
                fn(nd, nupts, neles, lin, gamma, up, ul, fp, fl, sp, sl, vp,
                   vl, upp, upl, stream)

        return Kernel(run, mats=[u, f, smats, verts, upts], misc=[gas],
                      name='tflux',
                      meta=dict(kind='tflux_euler', tplargs=tplargs,
                                dims=dims, u=u, f=f, smats=smats,
                                verts=verts, upts=upts,
                                geom_mode=lin))

    def _tflux_ns(self, tplargs, dims, extrns, u, f, gradu=None, smats=None,
                  rcpdjac=None, verts=None, upts=None, artvisc=None,
                  artvisc_vtx=None, gradwb=True):
        """``artvisc``: the artificial viscosity at the solution points
        (nupts, neles), when shock capturing is 'artificial-viscosity'
        (the vertex interpolation of pyfr/solvers/navstokes/kernels/
        tflux.mako:39-43, done by the avfill kernel).  ``artvisc_vtx`` is
        the argument of the reference's own elements (a view of the vertex
        values, None without artificial viscosity).  ``gradwb`` False
        leaves gradu in reference space (affine elements whose interface
        kernels transform the face gradients, ``facemet`` of intcflux)."""
        if artvisc_vtx is not None:
            raise NotImplementedError(
                'Artificial viscosity from vertex views: the b200 systems '
                'interpolate it to the points first (avfill)')
        av_on = tplargs.get('shock_capturing') == 'artificial-viscosity'
        if av_on != (artvisc is not None):
            raise ValueError('Artificial viscosity needs its field')
        # Unfused (flux anti-aliasing): f holds the physical gradient
        if ('fused' in tplargs.get('ktype', '')) != (gradu is not None):
            raise ValueError('The fused flux takes gradu, the unfused one '
                             'its gradient in f')

        nupts, neles = dims
        lin, (sp, sl), (rp, rl), (vp, vl), (upp, upl) = self._geom(
            tplargs, smats, rcpdjac, verts, upts)
        gas = _gas(tplargs['c'], tplargs.get('visc_corr', 'none'),
                   self.backend.ref_state)
        nd = tplargs['ndims']
        up, ul = _mat(u)
        fp, fl = _mat(f)
        gp, gl = _mat(gradu)

        if not gradwb and (gradu is None or artvisc is not None):
            raise ValueError('Leaving the gradient untransformed needs the '
                             'fused flux without artificial viscosity')
        if artvisc is not None:
            fn = self._fn('tflux_ns_av')
            ap, al = _mat(artvisc)

            def run(stream):
                fn(nd, nupts, neles, lin, C.byref(gas), up, ul, fp, fl, gp, gl,
                   sp, sl, rp, rl, vp, vl, upp, upl, ap, al, stream)
        else:
            fn = self._fn('tflux_ns' if gradwb else 'tflux_ns_refgrad')

            def run(stream):
                fn(nd, nupts, neles, lin, C.byref(gas), up, ul, fp, fl, gp, gl,
                   sp, sl, rp, rl, vp, vl, upp, upl, stream)

        return Kernel(run, mats=[u, f, gradu, smats, rcpdjac, verts, upts,
                                 artvisc],
                      misc=[gas], name='tflux',
                      meta=dict(kind='tflux_ns', tplargs=tplargs, dims=dims,
                                u=u, f=f, gradu=gradu, smats=smats,
                                rcpdjac=rcpdjac, verts=verts, upts=upts,
                                geom_mode=lin, gradwb=gradwb))

    def _wavespeed(self, tplargs, dims, extrns, u, wspd, smats=None,
                   rcpdjac=None, verts=None, upts=None):
        """Per-element largest wave speed in reference space
        (pyfr/solvers/euler/kernels/wavespeed.mako:9-44)."""
        nupts, neles = dims
        lin, (sp, sl), (rp, rl), (vp, vl), (upp, upl) = self._geom(
            tplargs, smats, rcpdjac, verts, upts)
        gas = _gas(tplargs['c'], 'none', self.backend.ref_state)
        fn, nd = self._fn('wavespeed'), tplargs['ndims']
        up, ul = _mat(u)
        wp = wspd.data

        def run(stream):
            fn(nd, nupts, neles, lin, C.byref(gas), up, ul, sp, sl, rp, rl, vp,
               vl, upp, upl, wp, stream)

        return Kernel(run, mats=[u, wspd, smats, rcpdjac, verts, upts],
                      misc=[gas], name='wavespeed',
                      meta=dict(kind='wavespeed', tplargs=tplargs, dims=dims,
                                u=u, wspd=wspd))

    def _gradcoru(self, tplargs, dims, extrns, gradu, smats=None,
                  rcpdjac=None, verts=None, upts=None):
        nupts, neles = dims
        lin, (sp, sl), (rp, rl), (vp, vl), (upp, upl) = self._geom(
            tplargs, smats, rcpdjac, verts, upts)
        fn, nd = self._fn('gradcoru'), tplargs['ndims']
        gp, gl = _mat(gradu)

        def run(stream):
            fn(nd, nupts, neles, lin, gp, gl, sp, sl, rp, rl, vp, vl, upp,
               upl, stream)

        return Kernel(run, mats=[gradu, smats, rcpdjac, verts, upts],
                      name='gradcoru',
                      meta=dict(kind='gradcoru', tplargs=tplargs, dims=dims,
                                gradu=gradu))

    def _source(self, tplargs, ploc, u):
        """The source macros of ``tplargs`` as a ``b200_src_t`` and the
        program matrix it points at, or (None, None) without any.  The one
        macro provided is the source plugin's (pyfr/plugins/source.py:8-31,
        pyfr/plugins/kernels/source.mako): src[i] += src_exprs[i]."""
        from pyfr_gb300.backend.lib import Src
        from pyfr_gb300.bcexpr import OPS, BCExpr, pack

        macros = [tuple(m) for m in tplargs.get('src_macros', [])]
        if not macros:
            return None, None
        if macros != [('pyfr.plugins.kernels.source', 'source')]:
            raise NotImplementedError(f'Source macros {macros} are not '
                                      'supported')
        if self.backend.ref_state is not None:
            raise NotImplementedError('Source terms take unshifted states')
        nd, nv = tplargs['ndims'], tplargs['nvars']
        exprs = list(tplargs['src_exprs'])
        if len(exprs) > nv or nv > 8:
            raise ValueError('More source terms than variables')
        progs, uses_x, uses_u = [], False, False
        for text in exprs:
            ex = BCExpr(str(text), nd, nv)
            if ex.const is not None:
                progs.append([(OPS['const'], ex.const)] if ex.const else [])
            else:
                progs.append(ex.prog)
            uses_x |= ex.uses_x
            uses_u |= ex.uses_u
        if uses_x and ploc is None:
            raise ValueError('Source terms of position need ploc')
        if uses_u and u is None:
            raise ValueError('Source terms of the solution need u')

        arr, spans = pack(progs)
        src = Src()
        for i, (start, n) in enumerate(spans):
            src.expr_start[i], src.expr_len[i] = start, n
        prog = None
        if len(arr):
            prog = self.backend.const_matrix(arr.view(np.int64)[None, :],
                                             dtype=np.int64)
            src.prog = prog.data
        if uses_x:
            src.ploc, src.ldp = _mat(ploc)
        if uses_u:
            src.u, src.ldu = _mat(u)
        return src, prog

    def _srcterms(self, mode, tplargs, dims, r, rcpdjac, ploc, u, tmat):
        """The source-term kernel in ``mode`` over r; the time is bound at
        run time (``t``) or read from element 1 of the device matrix
        ``tmat``."""
        src, prog = self._source(tplargs, ploc, u)
        nupts, neles = dims
        fn = self._fn('srcterms')
        nd, nv = tplargs['ndims'], tplargs['nvars']
        rp, rl = _mat(r)
        jp, jl = _mat(rcpdjac)
        if tmat is not None:
            src.t_dev = tmat.data + 8

        def run(stream, t=0.0):
            src.t = float(t)
            fn(mode, nd, nv, nupts, neles, rp, rl, jp, jl, C.byref(src),
               stream)

        mats = [r, rcpdjac, ploc, u, prog, tmat]
        return BindableKernel(run, ['t'], {'t': 0.0},
                              mats=[m for m in mats if m is not None],
                              misc=[src], name='srcterms',
                              meta=dict(kind='srcterms', mode=mode,
                                        tplargs=tplargs, dims=dims))

    def _negdivconf(self, tplargs, dims, extrns, tdivtconf, rcpdjac,
                    ploc=None, u=None, tmat=None, **kw):
        if tplargs.get('src_macros'):
            from pyfr_gb300.backend.lib import SRC_NEGDIVCONF
            k = self._srcterms(SRC_NEGDIVCONF, tplargs, dims, tdivtconf,
                               rcpdjac, ploc, u, tmat)
            if 't' in kw:
                k.bind(t=kw['t'])
            return k

        nupts, neles = dims
        fn, nv = self._fn('negdivconf'), tplargs['nvars']
        tp, tl = _mat(tdivtconf)
        rp, rl = _mat(rcpdjac)

        # `t` is accepted (and ignored) as the reference binds it at run time
        def run(stream, t=None):
            fn(nv, nupts, neles, tp, tl, rp, rl, stream)

        return BindableKernel(run, ['t'], {'t': kw.get('t', 0.0)},
                              mats=[tdivtconf, rcpdjac], name='negdivconf',
                              meta=dict(kind='negdivconf', tplargs=tplargs,
                                        dims=dims, tdivtconf=tdivtconf,
                                        rcpdjac=rcpdjac))

    def _addsrc(self, tplargs, dims, extrns, r, ploc=None, u=None,
                tmat=None, **kw):
        """R <- R + src: the source terms after an operator apply that
        already formed -(1/|J|) div F."""
        from pyfr_gb300.backend.lib import SRC_ADD
        k = self._srcterms(SRC_ADD, tplargs, dims, r, None, ploc, u, tmat)
        if 't' in kw:
            k.bind(t=kw['t'])
        return k

    def _evalsrcmacros(self, tplargs, dims, extrns, u, ploc=None,
                       tmat=None, **kw):
        if not tplargs.get('src_macros'):
            return NullKernel()
        from pyfr_gb300.backend.lib import SRC_EVAL
        k = self._srcterms(SRC_EVAL, tplargs, dims, u, None, ploc, u, tmat)
        if 't' in kw:
            k.bind(t=kw['t'])
        return k

    # ---- interface kernels ---------------------------------------------------

    def _intcflux_euler(self, tplargs, dims, extrns, ul, ur, nl):
        (n,) = dims
        rs = _rsolver(tplargs)
        fn, nd, gamma = (self._fn('intcflux_euler'), tplargs['ndims'],
                         tplargs['c']['gamma'])
        p_min = tplargs.get('p_min', P_MIN_DEFAULT)
        lb, lm, _ = _view(ul)
        rb, rm, _ = _view(ur)
        np_, nlp, nlu, nlm = self._normals(nl)
        ix64 = self._ix64
        gas = None

        if self.backend.ref_state is not None:
            if tplargs['rsolver'] != 'rusanov':
                raise NotImplementedError('The reference-state shift needs '
                                          'the Rusanov Riemann solver')
            fn = self._fn('intcflux_euler_shift')
            gas = _gas(tplargs['c'], 'none', self.backend.ref_state, p_min)

            def run(stream):
                fn(nd, n, C.byref(gas), lb, lm, rb, rm, ix64, np_, nlp, nlu,
                   stream)
        else:
            def run(stream):
                fn(nd, n, rs, gamma, p_min, lb, lm, rb, rm, ix64, np_, nlp,
                   nlu, stream)

        return Kernel(run, mats=[nl, nlm], views=[ul, ur], misc=[gas],
                      name='intcflux',
                      meta=dict(kind='intcflux_euler', tplargs=tplargs,
                                dims=dims, ul=ul, ur=ur, nl=nl))

    def _intcflux_ns(self, tplargs, dims, extrns, ul, ur, gradul, gradur, nl,
                     artvisc=None, facemet=None):
        """``facemet``: (metric matrix, left element columns, right element
        columns) when the face gradients are in reference space (the
        elements' flux kernel left them untransformed): the metric matrix
        holds S[i][j] of each affine element in row i*ndims + j and 1/|J|
        in the last row."""
        if (tplargs.get('shock_capturing') == 'artificial-viscosity') != \
                (artvisc is not None):
            raise ValueError('Artificial viscosity needs its field')
        if facemet is not None and artvisc is not None:
            raise ValueError('Face metrics and artificial viscosity do not '
                             'combine')

        (n,) = dims
        c = tplargs['c']
        rs = _rsolver(tplargs)
        if self.backend.ref_state is not None and tplargs['rsolver'] != 'rusanov':
            raise NotImplementedError('The reference-state shift needs the '
                                      'Rusanov Riemann solver')
        gas = _gas(c, tplargs.get('visc_corr', 'none'), self.backend.ref_state,
                   tplargs.get('p_min', P_MIN_DEFAULT))
        beta, tau = c['ldg-beta'], c['ldg-tau']
        fn, nd = self._fn('intcflux_ns'), tplargs['ndims']
        lb, lm, _ = _view(ul)
        rb, rm, _ = _view(ur)
        glb, glm, glr = _view(gradul)
        grb, grm, grr = _view(gradur)
        np_, nlp, nlu, nlm = self._normals(nl)
        ix64 = self._ix64

        if artvisc is not None:
            fn = self._fn('intcflux_ns_av')
            ab, am, _ = _view(artvisc)

            def run(stream):
                fn(nd, n, rs, C.byref(gas), beta, tau, lb, lm, rb, rm, glb,
                   glm, glr, grb, grm, grr, ix64, np_, nlp, nlu, ab, am,
                   stream)
        elif facemet is not None:
            fn = self._fn('intcflux_ns_refgrad')
            fm, fl_, fr_ = facemet
            fmp, fml = _mat(fm)

            def run(stream):
                fn(nd, n, rs, C.byref(gas), beta, tau, lb, lm, rb, rm, glb,
                   glm, glr, grb, grm, grr, ix64, np_, nlp, nlu, fmp, fml,
                   fl_.data, fr_.data, stream)
        else:
            def run(stream):
                fn(nd, n, rs, C.byref(gas), beta, tau, lb, lm, rb, rm, glb,
                   glm, glr, grb, grm, grr, ix64, np_, nlp, nlu, stream)

        return Kernel(run, mats=[nl, nlm] + list(facemet or ()),
                      views=[ul, ur, gradul, gradur] +
                      ([artvisc] if artvisc is not None else []),
                      misc=[gas], name='intcflux',
                      meta=dict(kind='intcflux_ns', tplargs=tplargs,
                                dims=dims, facemet=facemet is not None))

    # ---- boundary kernels -------------------------------------------------

    def _bc(self, tplargs, ploc=None):
        """(b200_bc_t, matrices it points at, run-time arguments) of a
        boundary kernel.  This package's own interfaces pass the struct
        ready (tplargs['bc']); PyFR's own interfaces pass the boundary type
        and its values in tplargs['c'] as numbers or as C expressions of
        ploc[i] and t (pyfr/solvers/baseadvec/inters.py:81-116), the
        coordinates as ``ploc``, and bind ``t`` (and, for the controlled
        characteristic boundaries, ``ic`` and ``im``,
        pyfr/solvers/euler/inters.py:108-215) at run time."""
        from pyfr_gb300.backend.lib import BC, BC_TYPES
        from pyfr_gb300.bcexpr import BCExpr, pack

        bc = tplargs.get('bc')
        if bc is not None:
            return bc, [], []
        bctype, c, nd = tplargs['bctype'], tplargs['c'], tplargs['ndims']
        if bctype not in BC_TYPES:
            raise NotImplementedError(f'Boundary type {bctype!r} is not '
                                      'provided')
        bc = BC(type=BC_TYPES[bctype])
        progs, fields = [], ['rho', 'p', 'u', 'v', 'w', 'cpTw']
        for f, k in enumerate(fields):
            v = c.get(k)
            if k in 'uvw' and 'uvw'.index(k) >= nd:
                v = None
            if v is None or k == 'cpTw':
                progs.append([])
                continue
            ex = BCExpr(str(v), nd)
            progs.append(ex.prog)
            val = ex.const if ex.const is not None else 0.0
            if k in 'uvw':
                bc.u['uvw'.index(k)] = val
            else:
                setattr(bc, k, val)
            if ex.uses_x and ploc is None:
                raise ValueError('Boundary expressions of position need '
                                 'ploc')
        bc.cpTw = float(c.get('cpTw', 0.0))
        bc.cpTt, bc.pt = float(c.get('cpTt', 0.0)), float(c.get('pt', 0.0))
        for i, v in enumerate(c.get('vc', [])):
            bc.vc[i] = float(v)

        mats, rt = [], ['t']
        if any(progs):
            arr, spans = pack(progs)
            prog = self.backend.const_matrix(arr.view(np.int64)[None, :],
                                             dtype=np.int64)
            bc.prog = prog.data
            for f, (start, n) in enumerate(spans):
                bc.expr_start[f], bc.expr_len[f] = start, n
            mats.append(prog)
            if ploc is not None:
                bc.ploc, bc.ldp = ploc.data, ploc.leaddim
                mats.append(ploc)
        if bctype in ('char-riem-inv-mass-flow', 'char-riem-inv-pressure'):
            rt += ['ic', 'im']
        return bc, mats, rt

    @staticmethod
    def _bc_kernel(run, bc, rt, **kw):
        """A boundary kernel whose struct takes the run-time arguments
        (the time, the controller's interpolation) before each launch."""
        def brun(stream, **args):
            for k, v in args.items():
                setattr(bc, k, float(v))
            run(stream)

        if not rt:
            return Kernel(run, **kw)
        return BindableKernel(brun, rt, {k: 0.0 for k in rt}, **kw)

    def _bccflux_euler(self, tplargs, dims, extrns, ul, nl, ploc=None,
                       **kw):
        (n,) = dims
        rs = _rsolver(tplargs)
        fn, nd, gamma = (self._fn('bccflux_euler'), tplargs['ndims'],
                         tplargs['c']['gamma'])
        p_min = tplargs.get('p_min', P_MIN_DEFAULT)
        bc, bmats, rt = self._bc(tplargs, ploc)
        lb, lm, _ = _view(ul)
        np_, nlp = _mat(nl)
        ix64 = self._ix64

        def run(stream):
            fn(nd, n, rs, gamma, p_min, C.byref(bc), lb, lm, ix64, np_, nlp,
               stream)

        return self._bc_kernel(run, bc, rt, mats=[nl] + bmats, views=[ul],
                               misc=[bc], name='bccflux',
                               meta=dict(kind='bccflux_euler',
                                         tplargs=tplargs, dims=dims))

    def _bcconu(self, tplargs, dims, extrns, ulin, ulout, nlin, ploc=None,
                **kw):
        (n,) = dims
        fn, nd, gamma = (self._fn('bcconu'), tplargs['ndims'],
                         tplargs['c']['gamma'])
        bc, bmats, rt = self._bc(tplargs, ploc)
        ib, im, _ = _view(ulin)
        ob, om, _ = _view(ulout)
        np_, nlp = _mat(nlin)
        ix64 = self._ix64

        def run(stream):
            fn(nd, n, gamma, C.byref(bc), ib, im, ob, om, ix64, np_, nlp,
               stream)

        return self._bc_kernel(run, bc, rt, mats=[nlin] + bmats,
                               views=[ulin, ulout], misc=[bc], name='bcconu',
                               meta=dict(kind='bcconu', dims=dims))

    def _bccflux_ns(self, tplargs, dims, extrns, ul, gradul, nl,
                    artvisc=None, ploc=None, **kw):
        if (tplargs.get('shock_capturing') == 'artificial-viscosity') != \
                (artvisc is not None):
            raise ValueError('Artificial viscosity needs its field')
        if self.backend.ref_state is not None:
            raise NotImplementedError('Boundaries take unshifted states')
        (n,) = dims
        c = tplargs['c']
        rs = _rsolver(tplargs)
        gas = _gas(c, tplargs.get('visc_corr', 'none'),
                   p_min=tplargs.get('p_min', P_MIN_DEFAULT))
        fn, nd = self._fn('bccflux_ns'), tplargs['ndims']
        bc, bmats, rt = self._bc(tplargs, ploc)
        lb, lm, _ = _view(ul)
        gb, gm, gr = _view(gradul)
        np_, nlp = _mat(nl)
        ix64 = self._ix64
        tau = c['ldg-tau']

        if artvisc is not None:
            fn = self._fn('bccflux_ns_av')
            ab, am, _ = _view(artvisc)

            def run(stream):
                fn(nd, n, rs, C.byref(gas), tau, C.byref(bc), lb, lm, gb, gm,
                   gr, ix64, np_, nlp, ab, am, stream)
        else:
            def run(stream):
                fn(nd, n, rs, C.byref(gas), tau, C.byref(bc), lb, lm, gb, gm,
                   gr, ix64, np_, nlp, stream)

        return self._bc_kernel(run, bc, rt, mats=[nl] + bmats,
                               views=[ul, gradul] +
                               ([artvisc] if artvisc is not None else []),
                               misc=[gas, bc], name='bccflux',
                               meta=dict(kind='bccflux_ns', dims=dims))

    def _mpiconu(self, tplargs, dims, extrns, ulin, urin, ulout,
                 urout=None):
        """The common solution at faces shared with another partition,
        written to this side only (pyfr/solvers/navstokes/kernels/
        mpiconu.mako:4-19): the two-sided kernel in its both-sides form
        with the received data as the right side and a scratch view (urout)
        for the other side's copy."""
        if urout is None:
            raise NotImplementedError('mpiconu needs a scratch view for the '
                                      'other side')
        return self._intconu(tplargs | {'both_sides': True}, dims, extrns,
                             ulin, urin, ulout, urout)

    def _mpicflux(self, tplargs, dims, extrns, ul, ur, nl, gradul=None,
                  gradur=None, artvisc=None):
        """The common flux at faces shared with another partition
        (pyfr/solvers/{euler,navstokes}/kernels/mpicflux.mako): the
        interface kernel with the received data, seen through a view, as
        its right side (which it also writes, unread)."""
        from pyfr_gb300.backend.types import View
        if not isinstance(ur, View):
            raise NotImplementedError('mpicflux reads the received data '
                                      'through a view')
        if gradul is None:
            return self._intcflux_euler(tplargs, dims, extrns, ul, ur, nl)
        return self._intcflux_ns(tplargs, dims, extrns, ul, ur, gradul,
                                 gradur, nl, artvisc=artvisc)

    def _intconu(self, tplargs, dims, extrns, ulin, urin, ulout, urout):
        (n,) = dims
        beta = tplargs['c']['ldg-beta']
        # both_sides: write the common solution to both sides (no prior
        # copy of the solution into the outputs is needed)
        name = 'intconu_both' if tplargs.get('both_sides') else 'intconu'
        fn, nv = self._fn(name), tplargs['nvars']
        a = [_view(v)[:2] for v in (ulin, urin, ulout, urout)]
        ix64 = self._ix64

        def run(stream):
            fn(nv, n, beta, *a[0], *a[1], *a[2], *a[3], ix64, stream)

        return Kernel(run, views=[ulin, urin, ulout, urout], name='intconu',
                      meta=dict(kind='intconu', tplargs=tplargs, dims=dims))

    # ---- integrator kernels ----------------------------------------------------

    def _rkvdh2(self, tplargs, dims, extrns, r1, r2, rold=None, rerr=None,
                dt=None, dtdev=None):
        """The rkvdh2 stage; with ``dtdev`` (a 1x1 FP64 matrix) the step
        size is read from device memory at run time, so that a captured
        step serves every dt and the bound dt is not used."""
        stage, nstages = tplargs['stage'], tplargs['nstages']
        errest = bool(tplargs['errest'])
        a = tplargs['a'][stage] if stage < nstages - 1 else 0.0
        b = tplargs['b'][stage]
        e = tplargs['e'][stage] if errest else 0.0
        n = r1.nrow*r1.leaddim
        p1, p2 = r1.data, r2.data
        po = rold.data if rold is not None else None
        pe = rerr.data if rerr is not None else None

        if dtdev is not None:
            fnd, pdt = self._fn('rkvdh2_dt'), dtdev.data

            def run(stream, dt):
                fnd(n, stage, nstages, int(errest), pdt, a, b, e, p1, p2, po,
                    pe, stream)
        else:
            fn = self._fn('rkvdh2')

            def run(stream, dt):
                fn(n, stage, nstages, int(errest), dt, a, b, e, p1, p2, po,
                   pe, stream)

        return BindableKernel(run, ['dt'], {'dt': dt if dt is not None
                                            else 0.0},
                              mats=[r1, r2, rold, rerr], name='rkvdh2',
                              meta=dict(kind='rkvdh2', tplargs=tplargs,
                                        dims=dims, r1=r1, r2=r2))


_BUILDERS = {
    'pyfr.solvers.euler.kernels.tflux': PointwiseKernelProvider._tflux_euler,
    'pyfr.solvers.navstokes.kernels.tflux': PointwiseKernelProvider._tflux_ns,
    'pyfr.solvers.baseadvecdiff.kernels.gradcoru':
        PointwiseKernelProvider._gradcoru,
    'pyfr.solvers.baseadvec.kernels.negdivconf':
        PointwiseKernelProvider._negdivconf,
    'pyfr.solvers.baseadvec.kernels.evalsrcmacros':
        PointwiseKernelProvider._evalsrcmacros,
    'pyfr_gb300.kernels.addsrc': PointwiseKernelProvider._addsrc,
    'pyfr.solvers.euler.kernels.intcflux':
        PointwiseKernelProvider._intcflux_euler,
    'pyfr.solvers.navstokes.kernels.intcflux':
        PointwiseKernelProvider._intcflux_ns,
    'pyfr.solvers.navstokes.kernels.intconu': PointwiseKernelProvider._intconu,
    'pyfr.solvers.navstokes.kernels.mpiconu': PointwiseKernelProvider._mpiconu,
    'pyfr.solvers.euler.kernels.mpicflux': PointwiseKernelProvider._mpicflux,
    'pyfr.solvers.navstokes.kernels.mpicflux':
        PointwiseKernelProvider._mpicflux,
    'pyfr.integrators.explicit.kernels.rkvdh2':
        PointwiseKernelProvider._rkvdh2,
    'pyfr.solvers.euler.kernels.wavespeed':
        PointwiseKernelProvider._wavespeed,
    'pyfr.solvers.euler.kernels.bccflux':
        PointwiseKernelProvider._bccflux_euler,
    'pyfr.solvers.navstokes.kernels.bcconu': PointwiseKernelProvider._bcconu,
    'pyfr.solvers.navstokes.kernels.bccflux':
        PointwiseKernelProvider._bccflux_ns,
}
