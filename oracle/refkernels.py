"""Recipe for ``oracle/_ref``: the reference's own pointwise kernels,
rendered from its ``.mako`` sources and compiled for the host.  Test
infrastructure only (it builds the checker, never the product).

The reference renders each kernel module with Mako and a backend-specific
kernel generator (``pyfr/backends/base/provider.py:74-101``,
``pyfr/backends/base/makoutil.py``).  Here the same module sources are
rendered by ``oracle/mako_lite.py`` with the reference's own
``makoutil`` helpers (macro expansion, ``pyfr.dot``, ``pyfr.array``...), and
a point generator of this package's own turns each ``<%pyfr:kernel>`` body
into a C function of one point whose arguments are that point's arrays,
plus a loop over ``n`` points.  The kernel bodies, and so every arithmetic
operation and its order, are the reference's text; gcc compiles them with
``-O2 -fno-fast-math -ffp-contract=off`` so that each operation is one IEEE
FP64 operation.

Sources are read from the reference checkout (``PYFR_REFERENCE``, default
``/root/reference``); outputs go to ``oracle/_ref/`` only.  The checkout is
only present where fixtures are made; ``tests/golden/make_pointwise.py``
evaluates the compiled kernels and commits their inputs and outputs as
``tests/golden/pointwise.npz``.
"""

import ctypes as C
import hashlib
import math
import os
import re
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, '_ref')


# ---- the standard set of rendered kernels (golden vectors, build) ----

GAMMA = 1.4
RSOLVERS = ['rusanov', 'hllc', 'hll', 'roe', 'roem', 'exact']

# RK45 (Kennedy-Carpenter 2N) coefficients as the reference states them
# (pyfr/integrators/explicit/steppers.py:218-243)
RK45_A = [970286171893 / 4311952581923, 6584761158862 / 12103376702013,
          2251764453980 / 15575788980749, 26877169314380 / 34165994151039]
RK45_B = [1153189308089 / 22510343858157, 1772645290293 / 4653164025191,
          -1672844663538 / 4480602732383, 2114624349019 / 3568978502595,
          5198255086312 / 14908931495163]
RK45_BHAT = [1016888040809 / 7410784769900, 11231460423587 / 58533540763752,
             -1563879915014 / 6823010717585, 606302364029 / 971179775848,
             1097981568119 / 3980877426909]


# A [solver-plugin-source] section exercising every kind of term the source
# plugin substitutes: coordinates, conserved variables, the time, a
# constant, abs and pi (pyfr/plugins/source.py:15-24)
SOURCE_OPTS = {'rho': '0.1*sin(x)*cos(y) + 0.01*t',
               'rhou': '-0.2*rhou*exp(-z*z) + pow(abs(rho), 0.5)',
               'rhov': 'mu*(x + y)/(1 + z*z) - 2*t*t',
               'rhow': 'min(rhov, y) - max(E, 0.5)*1e-3',
               'E': 'atan2(y, x)*t + tanh(E)*0.1 + pi/4'}
SOURCE_CONSTS = {'mu': '0.05'}
CONVARS3 = ['rho', 'rhou', 'rhov', 'rhow', 'E']


def _reference_module(name, relpath):
    """A module of the reference loaded from its file (importing it as a
    package member would run the package's __init__)."""
    import importlib.util
    if name not in sys.modules:
        path = os.path.join(reference_root(), relpath)
        spec = importlib.util.spec_from_file_location(name, path)
        mod = importlib.util.module_from_spec(spec)
        sys.modules[name] = mod
        spec.loader.exec_module(mod)
    return sys.modules[name]


def source_exprs(opts=SOURCE_OPTS, consts=SOURCE_CONSTS, convars=CONVARS3):
    """The source plugin's kernel expressions for ``opts``, made by the
    reference's own substitution (pyfr/plugins/source.py:15-24 with
    pyfr/inifile.py process_expr)."""
    process_expr = _reference_module('pyfr.inifile',
                                     'pyfr/inifile.py').process_expr
    subs = dict(consts)
    subs |= dict(x='ploc[0]', y='ploc[1]', z='ploc[2]')
    subs |= dict(abs='fabs', pi=math.pi)
    subs |= {v: f'u[{i}]' for i, v in enumerate(convars)}
    return [process_expr(opts[v], subs) for v in convars]


def constants(visc=False, sutherland=False, beta=0.5, tau=0.1):
    c = {'gamma': GAMMA}
    if visc:
        c |= {'mu': 0.05, 'Pr': 0.72, 'ldg-beta': beta, 'ldg-tau': tau}
        if sutherland:
            c |= {'cpTref': 3.0, 'cpTs': 1.2}
    return c


def standard_variants():
    """{cname: (module, kernel, tplargs, family)}."""
    v = {}
    for nd in (2, 3):
        nv = nd + 2
        base = dict(ndims=nd, nvars=nv, nverts=2**nd)
        v[f'euler{nd}_tflux'] = (
            'pyfr.solvers.euler.kernels.tflux', 'tflux',
            base | dict(c=constants(), ktype='curved'), f'euler{nd}_elem')
        v[f'euler{nd}_wavespeed'] = (
            'pyfr.solvers.euler.kernels.wavespeed', 'wavespeed',
            base | dict(c=constants(), ktype='curved'), f'euler{nd}_elem')
        for rs in RSOLVERS:
            v[f'euler{nd}_intcflux_{rs}'] = (
                'pyfr.solvers.euler.kernels.intcflux', 'intcflux',
                dict(ndims=nd, nvars=nv, rsolver=rs, c=constants(),
                     p_min=5*np.finfo(float).eps), f'euler{nd}_iface')
        for suth in (False, True):
            name = f'ns{nd}_tflux' + ('_suth' if suth else '')
            v[name] = (
                'pyfr.solvers.navstokes.kernels.tflux', 'tflux',
                base | dict(c=constants(True, suth), ktype='curved-fused',
                            visc_corr='sutherland' if suth else 'none',
                            shock_capturing='none'), f'ns{nd}_elem')
        combos = [(rs, b, t) for rs in ('rusanov', 'hllc')
                  for b in (0.5, 0.0, -0.5) for t in (0.1, 0.0)]
        combos += [(rs, 0.5, 0.1) for rs in ('hll', 'roe', 'roem', 'exact')]
        for rs, b, t in combos:
            name = f'ns{nd}_intcflux_{rs}_b{b:+.1f}_t{t:.1f}'
            v[name] = (
                'pyfr.solvers.navstokes.kernels.intcflux', 'intcflux',
                dict(ndims=nd, nvars=nv, rsolver=rs,
                     c=constants(True, beta=b, tau=t), visc_corr='none',
                     shock_capturing='none', p_min=5*np.finfo(float).eps),
                f'ns{nd}_iface')
        v[f'gradcoru{nd}'] = (
            'pyfr.solvers.baseadvecdiff.kernels.gradcoru', 'gradcoru',
            base | dict(ktype='curved'), f'ns{nd}_elem')
    for b in (0.5, 0.0, -0.5):
        v[f'intconu_b{b:+.1f}'] = (
            'pyfr.solvers.navstokes.kernels.intconu', 'intconu',
            dict(ndims=3, nvars=5, c=constants(True, beta=b)), 'conu')
    v['negdivconf'] = (
        'pyfr.solvers.baseadvec.kernels.negdivconf', 'negdivconf',
        dict(ndims=3, nvars=5, src_macros=[]), 'negdivconf')
    srctp = dict(ndims=3, nvars=5,
                 src_macros=[('pyfr.plugins.kernels.source', 'source')],
                 src_exprs=source_exprs())
    v['negdivconf_src'] = (
        'pyfr.solvers.baseadvec.kernels.negdivconf', 'negdivconf', srctp,
        'src')
    v['evalsrcmacros_src'] = (
        'pyfr.solvers.baseadvec.kernels.evalsrcmacros', 'evalsrcmacros',
        srctp, 'src')
    e = [b - bh for b, bh in zip(RK45_B, RK45_BHAT)]
    for errest in (False, True):
        for s in range(5):
            v[f'rkvdh2_s{s}_e{int(errest)}'] = (
                'pyfr.integrators.explicit.kernels.rkvdh2', 'rkvdh2',
                dict(nvars=5, stage=s, nstages=5, errest=errest, a=RK45_A,
                     b=RK45_B, e=e), 'rk')
    return v



def reference_root():
    return os.environ.get('PYFR_REFERENCE', '/root/reference')


def available():
    return os.path.isfile(os.path.join(reference_root(), 'pyfr', 'backends',
                                       'base', 'makoutil.py'))


# The backend "base" template of this checker: C99 on the host in FP64
_BASE = r"""<%namespace module='pyfr.backends.base.makoutil' name='pyfr'/>
#include <math.h>
#include <stdint.h>

#define min(a, b) ((a) < (b) ? (a) : (b))
#define max(a, b) ((a) > (b) ? (a) : (b))
#define PYFR_FP_PRECISE_BEGIN

typedef double fpdtype_t;
typedef int32_t ixdtype_t;

${next.body()}
"""


class _Arg:
    """One kernel argument from its specification string, e.g.
    ``'inout view fpdtype_t[5]'`` or ``'in broadcast-col view(8) fpdtype_t'``
    (the grammar of pyfr/backends/base/generator.py:8-32)."""

    def __init__(self, name, spec):
        self.name = name
        words = spec.split()
        self.intent = 'in'
        if words[0] in ('in', 'out', 'inout'):
            self.intent = words.pop(0)
        *attrs, last = words
        self.attrs = attrs
        m = re.fullmatch(r'([A-Za-z_]\w*)((?:\[\d+\])*)', last)
        if not m:
            raise ValueError(f'Bad argument specification {spec!r}')
        self.dtype = m[1]
        self.dims = [int(d) for d in re.findall(r'\d+', m[2])]
        vs = [int(re.search(r'\((\d+)\)', a)[1]) for a in attrs
              if a.startswith('view(')]
        self.viewstride = vs[0] if vs else 1
        self.isscalar = 'scalar' in attrs
        self.reduce = next((re.search(r'\((\w+)\)', a)[1] for a in attrs
                            if a.startswith('reduce(')), None)
        if self.viewstride > 1 and not self.dims:
            self.dims = [self.viewstride]
            self.viewstride = 1

    @property
    def ctype(self):
        return 'ixdtype_t' if self.dtype == 'ixdtype_t' else 'fpdtype_t'

    @property
    def size(self):
        return math.prod(self.dims) if self.dims else 1


class PointKernel:
    """Kernel generator for makoutil.kernel: C for one point plus a loop.

    ``void <cname>(long n, <vector args...>, <scalar args...>)``: vector
    arguments (sorted by name) are pointers to ``n`` consecutive per-point
    arrays of their declared shape; scalars are passed by value."""

    def __init__(self, name, ndim, args, body, fpdtype, ixdtype, *, cname):
        self.name = name
        self.cname = cname
        self.ndim = ndim
        self.body = body
        allargs = [_Arg(k, v) for k, v in sorted(args.items())]
        used = [a for a in allargs
                if re.search(rf'(?:^|[^\w]){a.name}\b', body)]
        self.vectargs = [a for a in used if not a.isscalar]
        self.scalargs = [a for a in used if a.isscalar]

    def argspec(self):
        return (self.ndim, [a.name for a in self.vectargs + self.scalargs],
                [a.dims for a in self.vectargs + self.scalargs])

    def render(self):
        params, pre, post, call = [], [], [], []
        for a in self.vectargs:
            if a.dims:
                decl = f'{a.ctype} {a.name}' + ''.join(f'[{d}]'
                                                       for d in a.dims)
                params.append(decl)
            else:
                params.append(f'{a.ctype} *_p_{a.name}')
                pre.append(f'{a.ctype} {a.name} = *_p_{a.name};')
                if a.intent != 'in':
                    post.append(f'*_p_{a.name} = {a.name};')
        for a in self.scalargs:
            params.append(f'{a.ctype} {a.name}')

        lines = [f'static void {self.cname}_point({", ".join(params)})',
                 '{', *pre, '{', self.body, '}', *post, '}', '']
        bparams = ['long _n']
        for a in self.vectargs:
            bparams.append(f'{a.ctype} *{a.name}')
            cast = ''.join(f'[{d}]' for d in a.dims[1:])
            if len(a.dims) > 1:
                call.append(f'({a.ctype} (*){cast})({a.name} + _i*{a.size})')
            else:
                call.append(f'{a.name} + _i*{a.size}')
        for a in self.scalargs:
            bparams.append(f'{a.ctype} {a.name}')
            call.append(a.name)
        lines += [f'void {self.cname}({", ".join(bparams)})', '{',
                  '    for (long _i = 0; _i < _n; _i++)',
                  f'        {self.cname}_point({", ".join(call)});', '}', '']
        return '\n'.join(lines)


def _makoutil(root):
    """The reference's ``pyfr/backends/base/makoutil.py``, loaded from its
    file: importing it as a package member would run
    ``pyfr/backends/__init__.py``, which needs the backends' dependencies."""
    import importlib.util
    name = 'pyfr.backends.base.makoutil'
    if name not in sys.modules:
        path = os.path.join(root, 'pyfr', 'backends', 'base', 'makoutil.py')
        spec = importlib.util.spec_from_file_location(name, path)
        mod = importlib.util.module_from_spec(spec)
        sys.modules[name] = mod
        spec.loader.exec_module(mod)
    return sys.modules[name]


def _lookup():
    from oracle import mako_lite
    root = reference_root()
    if root not in sys.path:
        sys.path.insert(0, root)
    mako_lite.install_runtime()
    makoutil = _makoutil(root)
    return mako_lite.Lookup(root, 'pyfr.backends.b200check.kernels',
                            overrides={'base': _BASE},
                            filters=[makoutil.mfilttag])


def render(mod, kname, cname, tplargs, extrns=None):
    """C source of kernel ``kname`` of module ``mod`` (e.g.
    'pyfr.solvers.euler.kernels.intcflux'), named ``cname``, together with
    its argument metadata."""
    from functools import partial
    specs = {}
    args = dict(fpdtype=np.float64, ixdtype=np.int32,
                fpdtype_max=float(np.finfo(np.float64).max), csubsz=1,
                soasz=1, math=math)
    args.update(tplargs)
    args['_kernel_generator'] = partial(_Recorder, cname=cname, out=specs)
    args['_macros'] = {}
    args['_extrns'] = dict(extrns or {})
    args['_kernel_argspecs'] = {}
    src = _lookup().render(mod, **args)
    if kname not in specs:
        raise ValueError(f'Kernel {kname!r} not defined in {mod}')
    return re.sub(r'\n\s*\n+', '\n\n', src), specs[kname]


class _Recorder(PointKernel):
    def __init__(self, *a, out, **kw):
        super().__init__(*a, **kw)
        out[self.name] = self


def _cident(name):
    """A C identifier for a variant name ('+' -> p, '-' -> m, '.' -> d)."""
    return re.sub(r'\W', '_', name.translate(str.maketrans('+-.', 'pmd')))


class RefLibrary:
    """A set of rendered kernels compiled into one shared object under
    ``oracle/_ref`` and called through ctypes."""

    def __init__(self, variants):
        """``variants``: {cname: (mod, kname, tplargs, extrns)}."""
        self.kernels = {}
        srcs = []
        for cname, (mod, kname, tplargs, extrns) in sorted(variants.items()):
            src, k = render(mod, kname, _cident(cname), tplargs, extrns)
            srcs.append(f'/* {cname}: {mod} */\n' +
                        src.split('typedef int32_t ixdtype_t;', 1)[1])
            self.kernels[cname] = k
        head = _BASE.split('${next.body()}')[0].split('\n', 1)[1]
        full = head + '\n'.join(srcs)
        os.makedirs(OUT, exist_ok=True)
        tag = hashlib.sha256(full.encode()).hexdigest()[:12]
        csrc = os.path.join(OUT, f'refkern_{tag}.c')
        so = os.path.join(OUT, f'librefkern_{tag}.so')
        if not os.path.exists(so):
            with open(csrc, 'w') as f:
                f.write(full)
            subprocess.run(['gcc', '-std=gnu11', '-O2', '-fPIC', '-shared',
                            '-fno-fast-math', '-ffp-contract=off', csrc,
                            '-o', so + '.tmp', '-lm'], check=True)
            os.replace(so + '.tmp', so)
        self.lib = C.CDLL(so)
        self.path = so

    def __call__(self, cname, n, **arrays):
        """Evaluate ``cname`` on ``n`` points.  Every vector argument is a
        float64 array of shape (n, *dims) (in/inout) and is updated in place
        for out/inout; missing outputs are allocated.  Returns the dict of
        all vector arrays after the call."""
        k = self.kernels[cname]
        fn = getattr(self.lib, _cident(cname))
        cargs, out = [C.c_long(n)], {}
        for a in k.vectargs:
            if a.name in arrays:
                x = np.ascontiguousarray(arrays[a.name], dtype=np.float64)
                x = x.reshape(n, *a.dims).copy()
            elif a.intent == 'in':
                raise KeyError(f'{cname}: missing input {a.name!r}')
            else:
                x = np.zeros((n, *a.dims))
            out[a.name] = x
            cargs.append(x.ctypes.data_as(C.c_void_p))
        for a in k.scalargs:
            cargs.append(C.c_double(float(arrays[a.name])))
        fn.restype = None
        fn(*cargs)
        return out


def standard_library():
    """The compiled library of the standard set of kernels."""
    return RefLibrary({k: (m, kn, tp, None)
                       for k, (m, kn, tp, _) in standard_variants().items()})
