"""PyFR's own host code driving the b200 backend (test infrastructure).

The reference's systems, interfaces, integrators and backend registry are
imported from its source tree -- ``baseline/_ref`` (a copy of the
reference's pure-Python package, made by ``__graft_entry__.build()``) or
the checkout named by ``PYFR_REFERENCE`` -- and run unmodified.  The
third-party modules it imports but does not use on this path are replaced
by stand-ins registered before the import: Mako and GiMMiK (kernel
sources: the b200 backend brings its own kernels), h5py (files: the mesh
is built in memory), pytools, platformdirs and rtree.  mpi4py is replaced
by a single-rank communicator whose collectives return their input.

Run as a script it advances a case with PyFR's integrator on the b200
backend and writes the solution:

  python -m tests.refstack --case vortex --n 8 --steps 5 --out soln.npz
"""

import argparse
import os
from pathlib import Path
import sys
import types

import numpy as np

ROOT = Path(__file__).resolve().parent.parent


def reference_tree():
    """Directory holding the reference's ``pyfr`` package, or None."""
    for p in (ROOT / 'baseline' / '_ref',
              Path(os.environ.get('PYFR_REFERENCE', '/root/reference'))):
        if (p / 'pyfr' / 'solvers' / 'base' / 'system.py').exists():
            return p
    return None


class _Comm:
    """A one-rank communicator: collectives return their input."""
    rank, size = 0, 1

    def bcast(self, obj, root=0):
        return obj

    def scatter(self, objs, root=0):
        return objs[0]

    def gather(self, obj, root=0):
        return [obj]

    def allgather(self, obj):
        return [obj]

    def allreduce(self, obj, op=None):
        return obj

    def reduce(self, obj, op=None, root=0):
        return obj

    def exscan(self, obj, op=None):
        # (undefined on the first rank: mpi4py returns None there)
        return None

    def Allreduce(self, sendbuf, recvbuf, op=None):
        src = sendbuf[0] if isinstance(sendbuf, (list, tuple)) else sendbuf
        dst = recvbuf[0] if isinstance(recvbuf, (list, tuple)) else recvbuf
        if src is not _InPlace:
            np.copyto(np.asarray(dst), np.asarray(src))

    def Reduce(self, sendbuf, recvbuf, op=None, root=0):
        self.Allreduce(sendbuf, recvbuf, op)

    def Bcast(self, buf, root=0):
        pass

    def Barrier(self):
        pass

    barrier = Barrier

    def Split(self, color=0, key=0):
        return self

    def Free(self):
        pass

    def free(self):
        pass

    @property
    def handle(self):
        return 0

    @staticmethod
    def fromhandle(h):
        return _Comm()


class _InPlaceType:
    pass


_InPlace = _InPlaceType()


class _Any:
    def __init__(self, *a, **k):
        pass

    def __call__(self, *a, **k):
        return _Any()

    def __getattr__(self, n):
        return _Any()

    def __mro_entries__(self, bases):
        return (object,)


def install_standins():
    """Register the stand-in modules (idempotent)."""
    if getattr(sys.modules.get('mpi4py'), '_b200_standin', False):
        return
    for name in ['platformdirs', 'mako', 'mako.lookup', 'mako.template',
                 'mako.runtime', 'mako.exceptions', 'h5py', 'gimmik',
                 'pytools', 'pytools.prefork', 'rtree', 'rtree.index',
                 'mpi4py', 'mpi4py.MPI', 'mpi4py.rc']:
        m = types.ModuleType(name)
        m.__getattr__ = lambda n: _Any()
        m.__path__ = []
        sys.modules[name] = m

    sys.modules['platformdirs'].user_cache_dir = lambda *a, **k: '/tmp/pyfrc'
    mpi = sys.modules['mpi4py.MPI']
    mpi.__file__ = 'libc.so.6'
    mpi.COMM_WORLD = _Comm()
    mpi.COMM_NULL = None
    mpi.IN_PLACE = _InPlace
    mpi.UNDEFINED = -32766
    for op in ('SUM', 'MAX', 'MIN', 'LOR', 'LAND', 'PROD'):
        setattr(mpi, op, op)
    mpi.Comm = _Comm
    mpi.Is_initialized = lambda: True
    mpi.Is_finalized = lambda: False
    sys.modules['mpi4py'].MPI = mpi
    sys.modules['mpi4py'].rc = sys.modules['mpi4py.rc']
    sys.modules['mpi4py']._b200_standin = True


def import_reference():
    """Import the reference package and register the b200 backend with its
    backend registry; returns the reference's ``pyfr`` module."""
    tree = reference_tree()
    if tree is None:
        raise RuntimeError('The reference source tree is not available')
    install_standins()
    if str(tree) not in sys.path:
        sys.path.insert(0, str(tree))
    import pyfr
    import pyfr.backends                      # noqa: F401
    import pyfr_gb300.backend.pyfr_plugin     # noqa: F401
    return pyfr


def reference_mesh(mesh):
    """The reference's in-memory ``Mesh`` (pyfr/readers/native.py:15-47) of
    a mesh made by ``pyfr_gb300.mesh``: vertices, and interfaces as
    connectivity over the codec entries 'eles/<type>/face/<n>'."""
    from pyfr.readers.native import Connectivity, Mesh
    from pyfr_gb300.shapes import SHAPES

    etypes = sorted(mesh.spts)
    bnames = sorted(getattr(mesh, 'bcon', {}))
    codec = [f'eles/{et}/face/{f}' for et in etypes
             for f in range(len(SHAPES[et].faces))]
    codec += [f'bc/{b}' for b in bnames]
    cidx = {c: i for i, c in enumerate(codec)}
    cidxmap = {i: (et, int(f)) for i, c in enumerate(codec)
               if c.startswith('eles/')
               for et, f in [c[5:].split('/face/')]}

    def con(side):
        c = np.array([cidx[f'eles/{et}/face/{f}']
                      for et, f in zip(side.etypes, side.fidxs)],
                     dtype=np.int16)
        return Connectivity(c, np.asarray(side.eidxs), cidxmap)

    lhs, rhs = mesh.con
    m = Mesh(fname='<memory>', raw=None, ndims=mesh.ndims, codec=codec,
             uuid='b200-memory-mesh', version=2, etypes=etypes,
             eidxs={et: np.arange(mesh.spts[et].shape[1]) for et in etypes},
             spts={et: mesh.spts[et] for et in etypes},
             spts_curved={et: np.zeros(mesh.spts[et].shape[1], bool)
                          for et in etypes},
             con=(con(lhs), con(rhs)), cidxmap=cidxmap,
             bcon={b: con(mesh.bcon[b]) for b in bnames})
    return m


def reference_cfg(cfg):
    """The case's configuration as the reference's Inifile."""
    from pyfr.inifile import Inifile
    return Inifile(cfg.tostr())


def run(case, n, steps, out=None, fake=False, source=False, single=False):
    """Advance ``case`` ('vortex' or 'tgv' on an n-cell mesh, or a
    boundary case 'bc-euler:<type>,<type>' / 'bc-ns:<type>,<type>' of
    ``tests/bc_cases.py``) by ``steps``
    RK45 steps with PyFR's own integrator on the b200 backend (with
    ``source``, and the case's [solver-plugin-source] terms through PyFR's
    own source plugin); returns the initial and final solutions, the step
    size and the integrator.  With ``single``: FP32 with split-BF16
    tensor-core operator applies and fused applies."""
    if fake:
        from tests import fake_lib
        fake_lib.install()
    import_reference()
    from pyfr.backends import get_backend
    from pyfr.solvers import get_solver
    from pyfr_gb300.cases import euler_vortex, ns_tgv

    lits = {}
    if case == 'vortex':
        cfg, mesh = euler_vortex(n=n, order=3, dt=1e-3)
    elif case.startswith('mixed-'):
        # 'mixed-<kinds>': a mixed box of pyfr_gb300.mesh.mixed_box (3-D
        # Euler density wave), the simplex point sets of this package
        # handed to the reference literally so that both order them alike
        from pyfr_gb300.cases import euler_mixed
        from pyfr_gb300.quadrules import point_set
        cfg, mesh = euler_mixed(n=n, kinds=case[6:], dt=1e-3)

        def lit(kind, rule):
            return ', '.join('(' + ', '.join(repr(float(x)) for x in q) + ')'
                             for q in point_set(kind, rule, 3))
        lits = {('solver-elements-tet', 'soln-pts'): lit('tet', 'alpha-opt'),
                ('solver-elements-pri', 'soln-pts'):
                    lit('pri', 'alpha-opt~gauss-legendre-lobatto'),
                ('solver-interfaces-tri', 'flux-pts'): lit('tri', 'alpha-opt')}
    elif case.startswith('bc-'):
        # 'bc-euler:<type>,<type>' or 'bc-ns:<type>,<type>'
        from tests.bc_cases import bc_case
        kind, types = case[3:].split(':')
        cfg, mesh, _ = bc_case(kind, types.split(','))
    else:
        cfg, mesh = ns_tgv(n=n, order=3, dt=1e-3)
    if source:
        from tests.oracle_util import add_source
        add_source(cfg, case)
    if single:
        cfg.set('backend', 'precision', 'single')
        cfg.set('backend-b200', 'mul-precision', 'bf16x3')
    rcfg = reference_cfg(cfg)
    for (sect, key), val in lits.items():
        rcfg.set(sect, key, val)
    rcfg.set('solver-time-integrator', 'tstart', '0.0')
    rcfg.set('solver-time-integrator', 'tend', repr(1e3))
    dt = rcfg.getfloat('solver-time-integrator', 'dt')

    backend = get_backend('b200', rcfg)
    solver = get_solver(backend, reference_mesh(mesh), None, rcfg)
    u0 = [np.array(s) for s in solver.soln]
    for _ in range(steps):
        solver.advance_to(solver.tcurr + dt)
    u1 = [np.array(s) for s in solver.soln]
    if out:
        ets = list(solver.system.ele_types)
        np.savez(out, u0=u0[0], u1=u1[0], dt=dt,
                 backend=type(backend).__mro__[1].__name__,
                 nsteps=solver.nacptsteps, etypes=np.array(ets),
                 **{f'u0/{et}': a for et, a in zip(ets, u0)},
                 **{f'u1/{et}': a for et, a in zip(ets, u1)})
    return u0, u1, dt, solver


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--case', default='vortex',
                    help="'vortex', 'tgv', 'mixed-<kinds>' or "
                         "'bc-euler|bc-ns:<type>,<type>'")
    ap.add_argument('--n', type=int, default=8)
    ap.add_argument('--steps', type=int, default=5)
    ap.add_argument('--out')
    ap.add_argument('--fake', action='store_true',
                    help='host logic only: the library stand-in, no GPU')
    ap.add_argument('--source', action='store_true',
                    help='with the case\'s [solver-plugin-source] terms')
    ap.add_argument('--single', action='store_true',
                    help='FP32 with split-BF16 tensor-core applies')
    ap.add_argument('--report', action='store_true',
                    help='print the kernels of the first RHS\'s graphs')
    a = ap.parse_args()
    _, _, _, solver = run(a.case, a.n, a.steps, a.out, a.fake, a.source,
                          a.single)
    if a.report:
        import json
        graphs = solver.system._rhs_graphs(0, 1)
        print(json.dumps([[k.name if k.name != 'mul' else
                           f"mul:{k.meta.get('impl')}" for k in g.klist]
                          for g in graphs]))


if __name__ == '__main__':
    sys.path.insert(0, str(ROOT))
    main()
