"""Ensembles of independent cases advanced together.

The batching form of the benchmark configurations: many independent 2-D
isentropic-vortex cases of uneven size, order and strength advanced in
lockstep.  Cases of the same order are merged into one mesh made of their
disjoint periodic boxes (no interface joins two cases, so the merged
system computes each case exactly as it would alone, element for element),
which turns many small launches into a few large ones: one system, and so
one launch per kernel, per order.  The RK steps of all the systems are
captured together as one CUDA graph per step.

The cases follow the reference's vortex initial condition
(``pyfr/solvers/euler/elements.py:86-129`` evaluating the ``[soln-ics]``
expressions of the isentropic vortex), each box translated so that the
cases do not overlap in space.
"""

import math

import numpy as np

from pyfr_gb300.cases import euler_vortex
from pyfr_gb300.mesh import Mesh, Side, periodic_box


def vortex_cases(ncases=64, seed=0, sizes=(16, 96), orders=(2, 3, 4),
                 betas=(2.0, 6.0)):
    """Draw the cases: side length (quads per direction) uniform in
    ``sizes``, order from ``orders`` and strength beta uniform in
    ``betas``, from one master seed (each case also records its own
    seed)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(ncases):
        out.append(dict(case=i, n=int(rng.integers(sizes[0], sizes[1] + 1)),
                        order=int(rng.choice(orders)),
                        beta=float(rng.uniform(*betas)),
                        seed=int(rng.integers(2**31))))
    return out


def _vortex_ics(ploc, beta, gamma=1.4, R=1.0, uinf=1.0, vinf=1.0):
    """Conserved variables of the vortex at points ploc (npts, 2, neles)
    centred at the origin of the box's own coordinates."""
    x, y = ploc[:, 0], ploc[:, 1]
    f = 1 - (x*x + y*y)/(R*R)
    rho = (1 - (gamma - 1)*beta*beta/(8*math.pi**2)*np.exp(f))**(1/(gamma - 1))
    u = uinf - beta/(2*math.pi)*(y/R)*np.exp(0.5*f)
    v = vinf + beta/(2*math.pi)*(x/R)*np.exp(0.5*f)
    p = rho**gamma/gamma
    E = p/(gamma - 1) + 0.5*rho*(u*u + v*v)
    return np.stack([rho, rho*u, rho*v, E], axis=1)


class EnsembleGroup:
    """All cases of one order merged into one mesh."""

    def __init__(self, order, cases, dt, precision, half=10.0, spacing=100.0):
        self.order, self.cases = order, cases
        spts, lt, le, lf, rt, re, rf = [], [], [], [], [], [], []
        self.slices = []
        off = 0
        for j, c in enumerate(cases):
            m = periodic_box('quad', c['n'], -half, half)
            s = m.spts['quad'].copy()
            s[..., 0] += spacing*j
            spts.append(s)
            lhs, rhs = m.con
            le.append(lhs.eidxs + off)
            lf.append(lhs.fidxs)
            re.append(rhs.eidxs + off)
            rf.append(rhs.fidxs)
            self.slices.append(slice(off, off + s.shape[1]))
            off += s.shape[1]
        self.neles = off
        nint = sum(len(x) for x in le)
        self.mesh = Mesh(ndims=2, spts={'quad': np.concatenate(spts, axis=1)},
                         con=(Side(['quad']*nint, np.concatenate(le),
                                   np.concatenate(lf)),
                              Side(['quad']*nint, np.concatenate(re),
                                   np.concatenate(rf))),
                         spts_curved={'quad': np.zeros(off, dtype=bool)},
                         periods=(2*half, 2*half))
        self.cfg, _ = euler_vortex(n=1, order=order, dt=dt,
                                   precision=precision, half=half)
        self.spacing = spacing

    def initial_solution(self, elements):
        """Per-case initial conditions at the solution points of the merged
        element set (each case with its own beta, in its own box)."""
        ploc = elements.ploc_at_np('upts')              # (nupts, 2, neles)
        u = np.empty((ploc.shape[0], 4, self.neles))
        for j, (c, sl) in enumerate(zip(self.cases, self.slices)):
            p = ploc[..., sl].copy()
            p[:, 0] -= self.spacing*j
            u[..., sl] = _vortex_ics(p, c['beta'])
        return u


class Ensemble:
    """Advance every group's system in lockstep with one CUDA graph per
    step; all groups share ``backend`` (one stream), whose precision
    the groups' configurations must name."""

    def __init__(self, backend, cases, dt, precision='double', mixed=False):
        from pyfr_gb300.integrators import MixedRKIntegrator, RKVdH2Integrator
        from pyfr_gb300.solvers.elements import EulerElements
        from pyfr_gb300.solvers.system import EulerSystem

        self.backend, self.dt = backend, dt
        byorder = {}
        for c in cases:
            byorder.setdefault(c['order'], []).append(c)
        self.groups = [EnsembleGroup(p, cs, dt, precision)
                       for p, cs in sorted(byorder.items())]

        icls = MixedRKIntegrator if mixed else RKVdH2Integrator
        self.intgs = []
        for g in self.groups:
            eles = EulerElements('quad', g.mesh.spts['quad'], g.cfg)
            ics = g.initial_solution(eles)
            self.intgs.append(icls(backend, EulerSystem, g.mesh, g.cfg,
                                   initsoln={'quad': ics}))
        self._graphs = {}
        self.nsteps = 0

    @property
    def gndofs(self):
        return sum(i.gndofs for i in self.intgs)

    @property
    def nstages(self):
        return self.intgs[0].nstages

    def step(self):
        be, stream = self.backend, self.backend.stream
        # The step size goes to each integrator's device copy (a no-op
        # after the first step)
        for i in self.intgs:
            i._set_dt(self.dt, stream)
        key = tuple(i.idxcurr for i in self.intgs)
        if key not in self._graphs:
            regs = []
            gexec = be.capture(
                lambda s: regs.extend(
                    i._enqueue_step(i.tcurr, self.dt, i.idxcurr, s)
                    for i in self.intgs), stream)
            self._graphs[key] = (gexec, regs)
        gexec, regs = self._graphs[key]
        be.lib.graph_launch(gexec, stream)
        for i, r in zip(self.intgs, regs):
            i.idxcurr = r[0]
            i.tcurr += self.dt
            i.nsteps += 1
            i.nrhsevals += i.nstages
        self.nsteps += 1

    def run_steps(self, n):
        for _ in range(n):
            self.step()
        self.backend.wait()

    def case_solutions(self):
        """Solution of every case, keyed by case number."""
        out = {}
        for g, i in zip(self.groups, self.intgs):
            (u,) = i.soln
            for c, sl in zip(g.cases, g.slices):
                out[c['case']] = u[..., sl]
        return out
