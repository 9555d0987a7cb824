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

import ctypes as C
import math
import weakref

import numpy as np

from pyfr_gb300.backend.types import Kernel

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

        # A solution read from a file restarts the run from its time, with
        # its configuration history and controller state
        # (pyfr/integrators/base.py:48-65)
        from pyfr_gb300.native import Solution
        self.isrestart = isinstance(initsoln, Solution)
        self._restart = initsoln if self.isrestart else None
        self.prevcfgs = {k: v.tostr() for k, v in
                         initsoln.prevcfgs.items()} if self.isrestart else {}
        if self.isrestart:
            initsoln = initsoln.data
        self.mesh_uuid = getattr(mesh, 'uuid', None)
        self.plugins = []
        self._plugin_times = []

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
        if self.controller not in ('none', 'pi', 'cfl'):
            raise ValueError(f'Unsupported controller {self.controller!r}')
        self.errest = self.controller == 'pi'
        self.needs_cfl = self.controller == 'cfl'
        nregs = 4 if self.errest else 2

        self._nregs = nregs
        self.system = self._make_system(backend, systemcls, mesh, initsoln,
                                        cfg)
        self.system.commit()
        self._setup_registers(initsoln)
        backend.commit()

        # Entropy filter: the starting minima (the integrator's preproc,
        # pyfr/integrators/explicit/base.py:39)
        for k in self.system.preproc_kernels(0):
            k.run(backend.stream)

        self.tstart = cfg.getfloat(sect, 'tstart', 0.0)
        self.tend = cfg.getfloat(sect, 'tend', None)
        self.tcurr = self._restart.stats.getfloat(sect, 'tcurr') \
            if self.isrestart else self.tstart

        # The reference's preproc prepares the boundary controllers once
        # before the first step (pyfr/integrators/explicit/base.py:39,
        # pyfr/solvers/base/system.py:435-439)
        for k in self.system.prepare_kernels(0, self.tcurr):
            k.run(backend.stream)
        # (the CFL controller computes its own first step size)
        self.dt = cfg.getfloat(sect, 'dt', 0.0) if self.needs_cfl else \
            cfg.getfloat(sect, 'dt')
        self.dtmin = cfg.getfloat(sect, 'dt-min', 1e-12)
        self.dtmax = cfg.getfloat(sect, 'dt-max', 1e2)
        self.idxcurr = 0
        self.nacptsteps = self.nrjctsteps = self.nsteps = 0
        self.dt_accepted = []
        self.nrhsevals = 0
        self._step_graphs = {}
        self._kcache = {}
        # (boundary controllers read the solution on the host before every
        # right-hand side, and partitions exchange face data through the
        # host, which a captured step cannot stop for)
        self.use_step_graph = backend.use_cuda_graphs and \
            not self.system.controlled_bcs and not self.system._mpi_inters

        # The step size lives in device memory (staged through page-locked
        # host memory), so that one captured graph per starting register
        # serves every dt the controller picks
        self._dt_dev = backend.matrix((1, 1), dtype=np.float64)
        backend.commit()
        self._dt_host = C.c_void_p()
        backend.lib.host_alloc(C.byref(self._dt_host), 8)
        weakref.finalize(self, backend.lib.host_free, self._dt_host.value)
        self._dt_evt = C.c_void_p()
        backend.lib.event_create(C.byref(self._dt_evt))
        weakref.finalize(self, backend.lib.event_destroy, self._dt_evt.value)
        self._dt_set = None

        # Boundary values that depend on the time: the step's start time
        # goes to device memory before each step (staged like dt) and a
        # one-thread kernel sets each stage's time t0 + c_i dt
        self._tdep = self.system.time_dependent
        if self._tdep:
            self._t_host = C.c_void_p()
            backend.lib.host_alloc(C.byref(self._t_host), 8)
            weakref.finalize(self, backend.lib.host_free, self._t_host.value)
            self._t_evt = C.c_void_p()
            backend.lib.event_create(C.byref(self._t_evt))
            weakref.finalize(self, backend.lib.event_destroy,
                             self._t_evt.value)
            self._t_pending = False
            self._tkerns = [self.system.stage_time_kernel(ci,
                                                          dt_dev=self._dt_dev)
                            for ci in self.c]

        if self.needs_cfl:
            # pyfr/integrators/controllers.py:7-38
            self._cfl = cfg.getfloat(sect, 'cfl')
            self._cfl_nsteps = cfg.getint(sect, 'cfl-nsteps', 1)
            self._order = cfg.getint('solver', 'order')

        if self.errest:
            self._rtol = cfg.getfloat(sect, 'rtol')
            convars = self.system.ele_map[self.system.ele_types[0]].convars
            atols = [cfg.getfloat(sect, f'atol-{v}', cfg.getfloat(sect, 'atol'))
                     for v in convars]
            # (tolerances are checked against the precision of the stored
            # solution, as pyfr/integrators/controllers.py:57-72 does)
            if self._rtol < 10*self.state_eps:
                raise ValueError('Relative tolerance too small')
            if any(a < 10*self.state_eps for a in atols):
                raise ValueError('Absolute tolerance too small')
            self._atols = atols
            self._saffac = cfg.getfloat(sect, 'safety-fact', 0.8)
            self._maxfac = cfg.getfloat(sect, 'max-fact', 1.1)
            self._minfac = cfg.getfloat(sect, 'min-fact', 0.9)
            self._pi_alpha = cfg.getfloat(sect, 'pi-alpha', 0.58)
            self._pi_beta = cfg.getfloat(sect, 'pi-beta', 0.42)
            self._errprev = 1.0
            self._ekerns = {}

            # Controller state of a restart; a change of tolerances resets
            # the previous error (pyfr/integrators/explicit/controllers.py:
            # 77-85)
            sd = self._restart.state.get('intg/ctrl') if self.isrestart \
                else None
            if sd is not None:
                self.dt, self._errprev = float(sd[0]), float(sd[1])
                old = self._restart.config
                keys = {k for c in (cfg, old) for k in c.items(sect)
                        if k.startswith(('atol', 'rtol'))}
                if any(cfg.get(sect, k, None) != old.get(sect, k, None)
                       for k in keys):
                    self._errprev = 1.0

    @property
    def gndofs(self):
        return self.system.gndofs

    # ---- plugins and output ------------------------------------------------

    def add_plugin(self, plugin):
        """Attach a solution plugin, called after every accepted step; a
        run that is not a restart calls it once at once (the initial
        output, pyfr/integrators/explicit/controllers.py:13-15)."""
        self.plugins.append(plugin)
        if not self.isrestart:
            self.backend.wait()
            plugin(self)

    def call_plugin_dt(self, tstart, dt):
        """Have ``advance_to`` land on tstart + k*dt (a plugin's output
        times, pyfr/integrators/base.py:254-270)."""
        self._plugin_times.append((tstart, dt))

    def _next_plugin_time(self):
        ts = [t0 + (math.floor((self.tcurr - t0)/dt + 1e-9) + 1)*dt
              for t0, dt in self._plugin_times]
        return min(ts, default=math.inf)

    def _run_plugins(self):
        if self.plugins:
            self.backend.wait()
            for p in self.plugins:
                p(self)

    @property
    def cfgmeta(self):
        """The configuration records of an output: ``config`` and the
        ``config-<n>`` chain (pyfr/integrators/base.py:369-381)."""
        cfg = self.cfg.tostr()
        n = len(self.prevcfgs)
        ret = dict(self.prevcfgs, config=cfg)
        if n == 0 or cfg != ret[f'config-{n - 1}']:
            ret[f'config-{n}'] = cfg
        return ret

    def collect_stats(self, stats):
        """Run statistics of an output (pyfr/integrators/base.py:328-
        348)."""
        sect = 'solver-time-integrator'
        stats.set(sect, 'tcurr', repr(self.tcurr))
        stats.set(sect, 'nacptsteps', self.nacptsteps)
        stats.set(sect, 'nrjctsteps', self.nrjctsteps)
        stats.set(sect, 'nsteps', self.nacptsteps + self.nrjctsteps)

    def serialise(self):
        """Serialised state restored by a restart."""
        if self.errest:
            return {'intg/ctrl': np.array([self.dt, self._errprev])}
        return {}

    def run(self):
        """Advance to the configured ``tend``."""
        if self.tend is None:
            raise ValueError('No tend in [solver-time-integrator]')
        self.advance_to(self.tend)

    def _make_system(self, backend, systemcls, mesh, initsoln, cfg):
        return systemcls(backend, mesh, initsoln, self._nregs, cfg,
                         needs_cfl=self.needs_cfl)

    def compute_dt_cfl(self):
        """Step size cfl/((2p + 1) max wave speed) of the current solution
        (pyfr/integrators/controllers.py:22-26)."""
        wmax = self.system.compute_max_wavespeed(self.idxcurr)
        wmax = float(self._allreduce([wmax], 'max')[0])
        return self._cfl/(wmax*(2*self._order + 1))

    def _allreduce(self, values, op='sum'):
        """``values`` combined over every partition of a partitioned
        system (through its exchanger), else as they are."""
        if not self.system._mpi_inters:
            return list(values)
        xchg = self.system.exchanger
        if xchg is None or not hasattr(xchg, 'allreduce'):
            raise NotImplementedError(
                'Step-size controllers across partitions need an exchanger '
                'with allreduce (one process per part: TorchExchanger)')
        return list(xchg.allreduce(values, op))

    def _global_error(self, local_sum):
        """The controller's error norm sqrt(sum / ndofs) over every
        partition (pyfr/integrators/controllers.py:105-117)."""
        tot, n = self._allreduce([local_sum, float(self.gndofs)])
        err = math.sqrt(tot/n)
        return err if not math.isnan(err) else 100

    def _setup_registers(self, initsoln):
        pass

    def _reject(self, iprev):
        self.idxcurr = iprev

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
                if self.use_step_graph:
                    kw['dtdev'] = self._dt_dev
                kerns.append(self.backend.kernel(
                    'rkvdh2', tplargs=tplargs, dims=[dims[0], dims[2]], **kw))
            self._kcache[key] = kerns
        return self._kcache[key]

    def _regs(self, idx):
        regs = list(range(4 if self.errest else 2))
        r1 = idx
        r2, *rs = [r for r in regs if r != r1]
        return r1, r2, rs

    def _time_kernels(self, i):
        return [self._tkerns[i]] if self._tdep else []

    def _set_t0(self, t, stream):
        """Enqueue the copy of the step's start time to device memory."""
        lib = self.backend.lib
        if self._t_pending:
            lib.event_sync(self._t_evt.value)
        C.c_double.from_address(self._t_host.value).value = t
        lib.memcpy_htod(self.system._tmat.data, self._t_host.value, 8,
                        stream)
        lib.event_record(self._t_evt.value, stream)
        self._t_pending = True

    def _prepare_kernels(self, ubank, i, t, dt):
        """The host steps before stage i's right-hand side (boundary
        controllers), at the stage time t + c_i dt."""
        if not self.system.controlled_bcs:
            return []
        if t is None:
            raise ValueError('Boundary controllers need the step time')
        return self.system.prepare_kernels(ubank, t + self.c[i]*dt)

    def step_kernels(self, idx, dt, t=None):
        """The kernels of one step starting from register ``idx`` at time
        ``t``, in launch order, and the resulting register indices."""
        r1, r2, rs = self._regs(idx)
        kl = []
        for i in range(self.nstages):
            kl.extend(self._time_kernels(i))
            kl.extend(self._prepare_kernels(r2 if i else r1, i, t, dt))
            for g in self.system.rhs_graphs(r2 if i else r1, r2):
                kl.extend(g.klist)
            for k in self._rk_kerns(i, r1, r2, *rs):
                k.bind(dt=dt)
                kl.append(k)
            r1, r2 = r2, r1
        # (the entropy filter's postproc of the new solution)
        kl.extend(self.system.postproc_kernels(r2))
        return kl, ((r2, *rs) if rs else (r2,))

    def _enqueue_step(self, t, dt, idx, stream):
        """Enqueue every stage of one step; returns the register indices."""
        kl, regs = self.step_kernels(idx, dt, t)
        for k in kl:
            k.run(stream)
        return regs

    def _set_dt(self, dt, stream):
        """Enqueue the copy of a new step size to device memory (a no-op
        while dt is unchanged)."""
        if dt != self._dt_set:
            lib = self.backend.lib
            # The staging buffer is reused once the previous copy has run
            if self._dt_set is not None:
                lib.event_sync(self._dt_evt.value)
            C.c_double.from_address(self._dt_host.value).value = dt
            lib.memcpy_htod(self._dt_dev.data, self._dt_host.value, 8, stream)
            lib.event_record(self._dt_evt.value, stream)
            self._dt_set = dt

    def step(self, t, dt):
        be, stream = self.backend, self.backend.stream
        if self._tdep:
            self._set_t0(t, stream)
            self._set_dt(dt, stream)
        if self.use_step_graph:
            self._set_dt(dt, stream)
            key = self.idxcurr
            if key not in self._step_graphs:
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
        return self._global_error(sum(k.retval[0] for k in ks))

    def advance_to(self, t):
        if t < self.tcurr:
            raise ValueError('Advance time is in the past')

        while self.tcurr < t - 1e-12*max(1.0, abs(t)):
            if self.needs_cfl and self.nacptsteps % self._cfl_nsteps == 0:
                self.dt = self.compute_dt_cfl()
            dt = min(self.dt, self.dtmax, t - self.tcurr,
                     self._next_plugin_time() - self.tcurr)
            if self.controller in ('none', 'cfl'):
                (idx,) = self.step(self.tcurr, dt)
                self.idxcurr = idx
                self.tcurr += dt
                self.nacptsteps += 1
                self.dt_accepted.append(dt)
                self._run_plugins()
                continue

            if self._pi_step(dt):
                self._run_plugins()

        self.backend.wait()

    def _pi_step(self, dt):
        """One attempted step of size dt under the PI controller
        (pyfr/integrators/explicit/controllers.py:87-125); returns whether
        it was accepted."""
        icurr, iprev, ierr = self.step(self.tcurr, dt)
        err = self._errest(icurr, ierr)
        expa = self._pi_alpha / self.stepper_order
        expb = self._pi_beta / self.stepper_order
        # (an exactly zero error, a steady solution, takes the largest
        # growth factor instead of dividing by zero)
        fac = max(err, 1e-300)**-expa * self._errprev**expb
        fac = min(self._maxfac, max(self._minfac, self._saffac*fac))
        self.dt = max(fac*dt, self.dtmin)

        if err < 1.0:
            self._errprev = err
            self.idxcurr = icurr
            self.tcurr += dt
            self.nacptsteps += 1
            self.dt_accepted.append(dt)
            return True

        if dt <= self.dtmin:
            raise RuntimeError('Minimum sized time step rejected')
        self._reject(iprev)
        self.nrjctsteps += 1
        return False

    def run_pi_steps(self, nsteps):
        """Take nsteps accepted steps under the PI controller (rejected
        attempts are retried with the reduced dt); returns the number of
        attempts."""
        if self.controller != 'pi':
            raise ValueError('run_pi_steps needs controller = pi')
        attempts = 0
        target = self.nacptsteps + nsteps
        while self.nacptsteps < target:
            if self._pi_step(min(self.dt, self.dtmax)):
                self._run_plugins()
            attempts += 1
        self.backend.wait()
        return attempts

    def run_steps(self, nsteps, dt=None):
        """Advance a fixed number of steps of size dt (default the
        configured dt) with the fixed-step controller."""
        dt = dt or self.dt
        for _ in range(nsteps):
            (idx,) = self.step(self.tcurr, dt)[:1]
            self.idxcurr = idx
            self.tcurr += dt
            self.nacptsteps += 1
            self._run_plugins()
        self.backend.wait()

    @property
    def state_eps(self):
        """Machine epsilon of the stored solution."""
        return self.backend.fpdtype_eps

    @property
    def soln(self):
        return self.system.ele_scal_upts(self.idxcurr)

    def _state_mats(self):
        return [m for bank in self.system.ele_banks for m in bank]

    def snapshot(self):
        """Device copies of every register, restored by ``restore``."""
        be, lib = self.backend, self.backend.lib
        snap = []
        for m in self._state_mats():
            c = be.matrix(m.ioshape, tags={'align'}, dtype=m.dtype)
            be.commit()
            lib.memcpy_dtod(c.data, m.data, m.nbytes, be.stream)
            snap.append(c)
        be.wait()
        return snap

    def restore(self, snap, release=True):
        be, lib = self.backend, self.backend.lib
        for m, c in zip(self._state_mats(), snap):
            lib.memcpy_dtod(m.data, c.data, m.nbytes, be.stream)
        be.wait()
        if release:
            for c in snap:
                be.free_matrix(c)


class MixedRKIntegrator(RKVdH2Integrator):
    """The chosen precision form: right-hand sides in FP32 (the system is
    built on a single-precision backend), the solution accumulated in FP64.

    The low-storage scheme's second register only ever carries the input
    of the next RHS evaluation, so it is kept in FP32 (system bank 0) and
    written by the stage kernel; system bank 1 receives the FP32 RHS; the
    solution itself (and the PI controller's error registers) are FP64.

    With a reference state the system works in q = T(u - u_ref) (the
    perturbation from u_ref with the energy replaced by dE - h_ref*drho,
    see ``b200_gas_t``), and the FP64 accumulator holds q: the stage kernel
    then forms the FP32 input with no FP64 arithmetic beyond its one FMA.
    ``soln`` maps q back to u.
    """

    def __init__(self, backend, systemcls, mesh, cfg, initsoln=None):
        if backend.fpdtype != np.float32:
            raise ValueError('The mixed-precision integrator needs a '
                             'single-precision backend')
        super().__init__(backend, systemcls, mesh, cfg, initsoln)

        # Entropy filter: the filter runs in FP32 on the system's copy of
        # the solution (the step's last stage leaves it there), and the
        # elements it changed go back to the FP64 solution; the starting
        # minima pass too (run by the base class) is merged here
        self._ef_merge = []
        if self.system._ef:
            ef = self.system._ef
            for j, (et, e) in enumerate(self.system.ele_map.items()):
                acc, u32, eff = self.acc[j], self.system.ele_banks[j][0], \
                    ef.ef_filter[et]
                args = (e.nupts, e.nvars, e.neles, eff.data, u32.data,
                        u32.leaddim, acc.data, acc.leaddim)

                def run(stream, args=args):
                    backend.lib.ef_merge_f64f32(*args, stream)

                self._ef_merge.append(Kernel(run, mats=[acc, u32, eff],
                                             name='ef_merge'))
            for k in self._ef_merge:
                k.run(backend.stream)
            backend.wait()

    def _make_system(self, backend, systemcls, mesh, initsoln, cfg):
        sysm = systemcls(backend, mesh, initsoln, 2, cfg,
                         needs_cfl=self.needs_cfl)

        if initsoln is not None:
            self._ics = [np.asarray(initsoln[et], dtype=np.float64)
                         for et in sysm.ele_types]
        else:
            self._ics = [e.set_ics_from_cfg() for e in sysm.ele_map.values()]

        # Reference-state shift of the FP32 right-hand side (Euler or
        # Navier-Stokes with the Rusanov solver, no boundaries or
        # partitions): the point means of rho, the momentum and p of the
        # initial condition.  Must be set before the kernels are built.
        self.uref, self.hs_ref = None, 0.0
        shift = cfg.get('backend-b200', 'reference-shift', 'auto')
        rs = cfg.get('solver-interfaces', 'riemann-solver')
        # (artificial viscosity senses the density itself and source terms
        # read the solution, so they keep the unshifted state, as
        # boundaries do)
        sc = cfg.get('solver', 'shock-capturing', 'none')
        if shift == 'auto' and sysm.name in ('navier-stokes', 'euler') and \
                rs == 'rusanov' and not sysm._bc_inters and sc == 'none' \
                and not sysm.has_src_macros and not sysm._mpi_inters:
            gamma = cfg.getfloat('constants', 'gamma')
            nd = sysm.ndims
            saved = self._restart.state.get('intg/uref') \
                if self.isrestart else None
            if saved is not None and len(saved) == nd + 3:
                # A restart keeps the run's reference state, so that it
                # continues bit for bit
                saved = np.asarray(saved, dtype=np.float64)
                rho_ref, mom, p_ref = float(saved[0]), saved[1:nd + 1].copy(), \
                    float(saved[nd + 2])
            else:
                cons = [np.concatenate([u[:, v].ravel() for u in self._ics])
                        for v in range(nd + 1)]
                pri = [e.con_to_pri(list(u.swapaxes(0, 1)), cfg)[-1]
                       for e, u in zip(sysm.ele_map.values(), self._ics)]
                p = np.concatenate([x.ravel() for x in pri])
                rho_ref, p_ref = float(cons[0].mean()), float(p.mean())
                mom = np.array([float(c.mean()) for c in cons[1:]])
                # A mean momentum at the rounding level of the state (a
                # flow with no mean motion) is taken as exactly zero, and
                # the Navier-Stokes kernels take a reference state at rest
                scale = max(float(np.sqrt(np.mean(c*c))) for c in cons[1:])
                if np.abs(mom).max() <= 1e-10*max(scale, 1e-300) or \
                        sysm.name == 'navier-stokes':
                    mom[:] = 0.0
            vref = mom/rho_ref
            e_ref = p_ref/(gamma - 1) + 0.5*rho_ref*float(vref @ vref)
            backend.ref_state = (rho_ref, p_ref, tuple(vref))
            self.uref = np.concatenate([[rho_ref], mom, [e_ref]])
            self.hs_ref = (e_ref + p_ref)/rho_ref
            self._ref_saved = np.concatenate([[rho_ref], mom, [e_ref, p_ref]])

        return sysm

    def _state_mats(self):
        mats = [m for bank in self.system.ele_banks for m in bank] + self.acc
        if self.errest:
            mats += self.rold + self.rerr
        return mats

    def _setup_registers(self, initsoln):
        be, sysm = self.backend, self.system
        ics = self._ics

        def reg(ic=None):
            return [be.matrix(ic_.shape, ic_ if ic is not None else None,
                              tags={'align'}, dtype=np.float64)
                    for ic_ in (ic if ic is not None else ics)]

        self.acc = reg([self.to_q(ic) for ic in ics])
        self.rold = reg() if self.errest else None
        self.rerr = reg() if self.errest else None
        be.commit()
        self.refresh_input(be.stream)
        be.wait()

    def serialise(self):
        """The base state and, with the reference-state transform, the
        reference state itself (rho, momentum, E and p), which a restart
        keeps."""
        out = super().serialise()
        if self.uref is not None:
            out['intg/uref'] = self._ref_saved.copy()
        return out

    @property
    def state_eps(self):
        # The solution and the error registers are FP64
        return float(np.finfo(np.float64).eps)

    def to_q(self, u):
        """Solution (nupts, nvars, neles) -> the integrated variables."""
        if self.uref is None:
            return np.asarray(u, dtype=np.float64)
        q = u - self.uref[None, :, None]
        q[:, -1] -= self.hs_ref*q[:, 0]
        return q

    def from_q(self, q):
        if self.uref is None:
            return q
        u = q + self.uref[None, :, None]
        u[:, -1] += self.hs_ref*q[:, 0]
        return u

    def refresh_input(self, stream):
        """Enqueue the FP32 RHS input from the FP64 accumulator (which
        holds q when there is a reference state)."""
        lib = self.backend.lib
        for j, bank in enumerate(self.system.ele_banks):
            acc = self.acc[j]
            lib.cast_f64_f32(acc.nrow*acc.leaddim, acc.data, bank[0].data,
                             0, None, stream)

    def _stage_kernel(self, i, j, dt):
        lib, nst, errest = self.backend.lib, self.nstages, int(self.errest)
        bank, acc = self.system.ele_banks[j], self.acc[j]
        n = acc.nrow*acc.leaddim
        a = self.a[i] if i < nst - 1 else 0.0
        b = self.b[i]
        e = self.e[i] if self.errest else 0.0
        ro = self.rold[j].data if self.errest else None
        re = self.rerr[j].data if self.errest else None
        pa, pr, pu = acc.data, bank[1].data, bank[0].data

        if self.use_step_graph:
            pdt = self._dt_dev.data

            def run(stream):
                lib.rkmixed_dt_f64f32(n, i, nst, errest, pdt, a, b, e, pa, pr,
                                      pu, ro, re, stream)
        else:
            def run(stream):
                lib.rkmixed_f64f32(n, i, nst, errest, dt, a, b, e, pa, pr,
                                   pu, ro, re, stream)

        return Kernel(run, mats=[acc, bank[0], bank[1]], name='rkmixed',
                      meta=dict(kind='rkmixed', n=n))

    def _fuse_stage(self, rhs, i, dt):
        """Move the stage update of each element type into the epilogue of
        the apply that writes its right-hand side (the fused divergence,
        correction and negdivconf), when that apply is the last kernel to
        touch it: R then never goes to memory.  Returns the kernel list and
        the element types done."""
        be, sysm = self.backend, self.system
        if not be.fuse_stage or self.errest or sysm._ef:
            return rhs, set()
        tc = next((p for p in be._providers
                   if hasattr(p, 'with_stage')), None)
        nst = self.nstages
        a = self.a[i] if i < nst - 1 else 0.0
        dtdev = self._dt_dev if self.use_step_graph else None
        out, done = list(rhs), set()
        for j, bank in enumerate(sysm.ele_banks):
            r = bank[1]
            idx = [n for n, k in enumerate(out)
                   if any(m is r for m in getattr(k, 'mats', ()))]
            if not idx:
                continue
            k = out[idx[-1]]
            if k.name != 'mul' or k.meta.get('out') is not r or \
                    sum(1 for n in idx if out[n].meta.get('out') is r) != 1:
                continue
            kk = tc.with_stage(k, self.acc[j], bank[0], a, self.b[i],
                               i == nst - 1, dt=dt, dtdev=dtdev)
            if kk is not None:
                out[idx[-1]] = kk
                done.add(j)
        return out, done

    def step_kernels(self, idx, dt, t=None):
        kl = []
        for i in range(self.nstages):
            kl.extend(self._time_kernels(i))
            kl.extend(self._prepare_kernels(0, i, t, dt))
            rhs = [k for g in self.system.rhs_graphs(0, 1) for k in g.klist]
            rhs, done = self._fuse_stage(rhs, i, dt)
            kl.extend(rhs)
            kl.extend(self._stage_kernel(i, j, dt)
                      for j in range(len(self.acc)) if j not in done)
        # (the entropy filter of the new solution, merged back into FP64)
        post = self.system.postproc_kernels(0)
        if post:
            kl.extend(post)
            kl.extend(self._ef_merge)
        return kl, ((0, 1, 2) if self.errest else (0,))

    def _reject(self, iprev):
        self._restore_previous()

    def _restore_previous(self):
        lib, stream = self.backend.lib, self.backend.stream
        for j in range(len(self.acc)):
            acc = self.acc[j]
            lib.memcpy_dtod(acc.data, self.rold[j].data, acc.nbytes, stream)
        self.refresh_input(stream)

    def _errest(self, icurr, ierr):
        if 'mixed' not in self._ekerns:
            self._ekerns['mixed'] = [
                self.backend.kernel('errest', a, r, self._atols,
                                    uref=self.uref, hcoef=self.hs_ref)
                for a, r in zip(self.acc, self.rerr)]
        ks = self._ekerns['mixed']
        for k in ks:
            k.bind(rtol=self._rtol)
            k.run(self.backend.stream)
        self.backend.wait()
        return self._global_error(sum(k.retval[0] for k in ks))

    @property
    def soln(self):
        return [self.from_q(a.get()) for a in self.acc]
