"""Explicit low-storage Runge-Kutta time integration.

``RKVdH2Integrator`` is the two-register (four with an error estimate)
scheme of ``pyfr/integrators/explicit/steppers.py:111-243`` (rk34 and rk45
coefficients) driven by the 'none' (fixed dt) or 'pi' (adaptive)
controller (``pyfr/integrators/explicit/controllers.py:27-125``,
``pyfr/integrators/controllers.py:40-117``).  The GDoF/s statistic is the
reference's ``gndofs * nrhsevals / walltime``
(``pyfr/integrators/base.py:348-349``).

When CUDA graphs are enabled the whole step (every stage's RHS graphs and
stage kernels) is captured once per starting register and replayed with a
single launch.
"""

import math
import time

import numpy as np

RK_COEFFS = {
    'rk45': dict(
        order=4,
        a=[970286171893 / 4311952581923, 6584761158862 / 12103376702013,
           2251764453980 / 15575788980749, 26877169314380 / 34165994151039],
        b=[1153189308089 / 22510343858157, 1772645290293 / 4653164025191,
           -1672844663538 / 4480602732383, 2114624349019 / 3568978502595,
           5198255086312 / 14908931495163],
        bhat=[1016888040809 / 7410784769900, 11231460423587 / 58533540763752,
              -1563879915014 / 6823010717585, 606302364029 / 971179775848,
              1097981568119 / 3980877426909]),
    'rk34': dict(
        order=3,
        a=[11847461282814 / 36547543011857, 3943225443063 / 7078155732230,
           -346793006927 / 4029903576067],
        b=[1017324711453 / 9774461848756, 8237718856693 / 13685301971492,
           57731312506979 / 19404895981398, -101169746363290 / 37734290219643],
        bhat=[15763415370699 / 46270243929542, 514528521746 / 5659431552419,
              27030193851939 / 9429696342944, -69544964788955 / 30262026368149]),
}


class RKVdH2Integrator:
    def __init__(self, backend, systemcls, mesh, cfg, initsoln=None):
        self.backend = backend
        self.cfg = cfg

        sect = 'solver-time-integrator'
        self.scheme = cfg.get(sect, 'scheme', 'rk45')
        if self.scheme not in RK_COEFFS:
            raise ValueError(f'Unsupported scheme {self.scheme!r}')
        co = RK_COEFFS[self.scheme]
        self.a, self.b, self.bhat = co['a'], co['b'], co['bhat']
        self.stepper_order = co['order']
        self.c = [0.0] + [sum(self.b[:i]) + ai for i, ai in enumerate(self.a)]
        self.e = [b - bh for b, bh in zip(self.b, self.bhat)]
        self.nstages = len(self.c)

        self.controller = cfg.get(sect, 'controller', 'none')
        if self.controller not in ('none', 'pi'):
            raise ValueError(f'Unsupported controller {self.controller!r}')
        self.errest = self.controller == 'pi'
        nregs = 4 if self.errest else 2

        self.system = systemcls(backend, mesh, initsoln, nregs, cfg)
        self.system.commit()
        backend.commit()

        self.tcurr = cfg.getfloat(sect, 'tstart', 0.0)
        self.dt = cfg.getfloat(sect, 'dt')
        self.dtmin = cfg.getfloat(sect, 'dt-min', 1e-12)
        self.dtmax = cfg.getfloat(sect, 'dt-max', 1e2)
        self.idxcurr = 0
        self.nacptsteps = self.nrjctsteps = self.nsteps = 0
        self.nrhsevals = 0
        self._step_graphs = {}
        self._kcache = {}
        self.use_step_graph = backend.use_cuda_graphs

        if self.errest:
            self._rtol = cfg.getfloat(sect, 'rtol')
            convars = self.system.ele_map[self.system.ele_types[0]].convars
            atols = [cfg.getfloat(sect, f'atol-{v}', cfg.getfloat(sect, 'atol'))
                     for v in convars]
            if any(a < 10*backend.fpdtype_eps for a in atols):
                raise ValueError('Absolute tolerance too small')
            self._atols = atols
            self._saffac = cfg.getfloat(sect, 'safety-fact', 0.8)
            self._maxfac = cfg.getfloat(sect, 'max-fact', 1.1)
            self._minfac = cfg.getfloat(sect, 'min-fact', 0.9)
            self._pi_alpha = cfg.getfloat(sect, 'pi-alpha', 0.58)
            self._pi_beta = cfg.getfloat(sect, 'pi-beta', 0.42)
            self._errprev = 1.0
            self._ekerns = {}

    @property
    def gndofs(self):
        return self.system.gndofs

    # ---- one step ----------------------------------------------------------

    def _rk_kerns(self, stage, r1, r2, rold=None, rerr=None):
        key = (stage, r1, r2, rold, rerr)
        if key not in self._kcache:
            self.backend.pointwise.register(
                'pyfr.integrators.explicit.kernels.rkvdh2')
            tplargs = dict(a=self.a, b=self.b, e=self.e, stage=stage,
                           nstages=self.nstages, nvars=self.system.nvars,
                           errest=rold is not None)
            kerns = []
            for dims, em in zip(self.system.ele_shapes.values(),
                                self.system.ele_banks):
                kw = dict(r1=em[r1], r2=em[r2])
                if rold is not None:
                    kw |= dict(rold=em[rold], rerr=em[rerr])
                kerns.append(self.backend.kernel(
                    'rkvdh2', tplargs=tplargs, dims=[dims[0], dims[2]], **kw))
            self._kcache[key] = kerns
        return self._kcache[key]

    def _regs(self, idx):
        regs = list(range(4 if self.errest else 2))
        r1 = idx
        r2, *rs = [r for r in regs if r != r1]
        return r1, r2, rs

    def _enqueue_step(self, t, dt, idx, stream):
        """Enqueue every stage of one step; returns the register indices."""
        r1, r2, rs = self._regs(idx)
        for i, ci in enumerate(self.c):
            for g in self.system.rhs_graphs(r2 if i else r1, r2):
                for k in g.klist:
                    k.run(stream)
            for k in self._rk_kerns(i, r1, r2, *rs):
                k.bind(dt=dt)
                k.run(stream)
            r1, r2 = r2, r1
        return (r2, *rs) if rs else (r2,)

    def step(self, t, dt):
        be, stream = self.backend, self.backend.stream
        if self.use_step_graph:
            key = (self.idxcurr, dt)
            if key not in self._step_graphs:
                # Retire graphs captured for another dt
                for k in [k for k in self._step_graphs if k[1] != dt]:
                    be.release_gexec(self._step_graphs.pop(k)[0])
                res = []
                gexec = be.capture(
                    lambda s: res.append(self._enqueue_step(t, dt,
                                                            self.idxcurr, s)),
                    stream)
                self._step_graphs[key] = (gexec, res[0])
            gexec, regs = self._step_graphs[key]
            be.lib.graph_launch(gexec, stream)
        else:
            regs = self._enqueue_step(t, dt, self.idxcurr, stream)

        self.nrhsevals += self.nstages
        self.nsteps += 1
        return regs

    # ---- time loop -----------------------------------------------------------

    def _errest(self, icurr, ierr):
        key = (icurr, ierr)
        if key not in self._ekerns:
            self._ekerns[key] = [
                self.backend.kernel('errest', em[icurr], em[ierr],
                                    self._atols)
                for em in self.system.ele_banks]
        ks = self._ekerns[key]
        for k in ks:
            k.bind(rtol=self._rtol)
            k.run(self.backend.stream)
        self.backend.wait()
        err = math.sqrt(sum(k.retval[0] for k in ks) / self.gndofs)
        return err if not math.isnan(err) else 100

    def advance_to(self, t):
        if t < self.tcurr:
            raise ValueError('Advance time is in the past')

        while self.tcurr < t - 1e-12*max(1.0, abs(t)):
            dt = min(self.dt, self.dtmax, t - self.tcurr)
            if self.controller == 'none':
                (idx,) = self.step(self.tcurr, dt)
                self.idxcurr = idx
                self.tcurr += dt
                self.nacptsteps += 1
                continue

            icurr, iprev, ierr = self.step(self.tcurr, dt)
            err = self._errest(icurr, ierr)
            expa = self._pi_alpha / self.stepper_order
            expb = self._pi_beta / self.stepper_order
            fac = err**-expa * self._errprev**expb
            fac = min(self._maxfac, max(self._minfac, self._saffac*fac))
            self.dt = max(fac*dt, self.dtmin)

            if err < 1.0:
                self._errprev = err
                self.idxcurr = icurr
                self.tcurr += dt
                self.nacptsteps += 1
            else:
                if dt <= self.dtmin:
                    raise RuntimeError('Minimum sized time step rejected')
                self.idxcurr = iprev
                self.nrjctsteps += 1

        self.backend.wait()

    def run_steps(self, nsteps, dt=None):
        """Advance a fixed number of steps of size dt (default the
        configured dt) with the fixed-step controller."""
        dt = dt or self.dt
        for _ in range(nsteps):
            (idx,) = self.step(self.tcurr, dt)[:1]
            self.idxcurr = idx
            self.tcurr += dt
        self.backend.wait()

    @property
    def soln(self):
        return self.system.ele_scal_upts(self.idxcurr)
