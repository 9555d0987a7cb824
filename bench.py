"""Benchmark: GDoF/s per RHS evaluation of the flux-reconstruction solver.

Workload (N=1): 3-D compressible Navier-Stokes Taylor-Green vortex,
periodic [-pi, pi]^3, 48^3 hexahedra, p=3 Gauss-Legendre points (64 per
element, 5 variables, 35.4 M DoF), Rusanov + LDG, RK45 fixed dt, plain
FP64.  One step = one RK45 step (5 RHS evaluations + 5 stage updates).
GDoF/s = gndofs * nrhs / time, the reference's rhs-gdof/s statistic.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

--impl reference times the CPU restatement of the reference's algorithm
(the oracle) on the host cores, on a bounded sample of the same workload.
Under torchrun each rank runs an independent replica (the path is not
partitioned across GPUs); value aggregates all ranks.
"""

import argparse
import json
import math
import os
import resource
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = ('GDoF/s per RHS eval: FP64 plain vs split-BF16/FP32 form at L2 err '
          '≤1e-6, 1 GB300')


def _peaks():
    p = ROOT / 'MEASURED_PEAKS.json'
    if p.exists():
        d = json.loads(p.read_text())
        return d['hbm_gbs'], 'measured'
    return 6800.0, 'fallback'


# ---------------------------------------------------------------------------
# Clock sampling
# ---------------------------------------------------------------------------

class ClockSampler:
    Q = ('clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,'
         'clocks_event_reasons.hw_thermal_slowdown,'
         'clocks_event_reasons.sw_thermal_slowdown,'
         'clocks_event_reasons.sw_power_cap')

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ['nvidia-smi', f'--id={self.index}', f'--query-gpu={self.Q}',
                 '--format=csv,noheader,nounits', '-lms', '200'],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self._t.join(timeout=2)

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown',
                 'sw_power_cap']
        for l in self.lines:
            f = [x.strip() for x in l.split(',')]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                smax = float(f[1])
            except ValueError:
                continue
            for n, v in zip(names, f[3:7]):
                if v.lower() == 'active':
                    reasons.add(n)
        if not sm:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': [],
                    'samples': 0}
        return {'sm_mhz': statistics.median(sm), 'sm_max_mhz': smax,
                'reasons': sorted(reasons), 'samples': len(sm)}


# ---------------------------------------------------------------------------
# Algorithmic bytes of each kernel launch (FP64 unless noted)
# ---------------------------------------------------------------------------

def kernel_bytes(k, be):
    m = k.meta
    kind = m.get('kind', k.name)
    itemsize = 8 if be.fpdtype == np.float64 else 4
    if k.name == 'mul':
        # out = alpha*S*(A@B [+ A2@B2]) + beta*out over nbatch slices:
        # read B (and B2), write out (and read it when beta = 1), read S
        a, b, out = m['a'], m['b'], m['out']
        ncol, nb = b.ncol, m.get('nbatch', 1)
        kin = a.ncol + (m['a2'].ncol if m.get('a2') is not None else 0)
        nout = a.nrow*ncol*(2 if m['beta'] else 1)
        if m.get('rk_stage'):
            # RK stage in the epilogue: the output is not stored; the FP64
            # solution is read and written and the FP32 input written
            nout = a.nrow*ncol*(8 + 8 + 4)//itemsize
        rs = m.get('rowscale')
        srows = rs.nrow*rs.ncol if rs is not None else 0
        return (nb*(kin*ncol + nout) + srows)*itemsize
    if kind in ('tflux_ns', 'tflux_euler'):
        nupts, neles = m['dims']
        nd, nv = m['tplargs']['ndims'], m['tplargs']['nvars']
        # u in and F out; the NS flux also reads the gradient and, unless
        # it leaves it in reference space, writes it back transformed
        per_pt = nv + nd*nv
        if kind == 'tflux_ns':
            per_pt += nd*nv*(2 if m.get('gradwb', True) else 1)
        # Metric terms (nd*nd + 1 values) stored per point or, for affine
        # elements, per element; or the vertices they are rebuilt from
        geo = {1: (2**nd)*nd*neles, 2: neles*(nd*nd + 1)}.get(
            m.get('geom_mode'), nupts*neles*(nd*nd + 1))
        return (per_pt*nupts*neles + geo)*itemsize
    if kind in ('intcflux_ns', 'intcflux_euler'):
        (n,) = m['dims']
        nd, nv = m['tplargs']['ndims'], m['tplargs']['nvars']
        # Gradients are read from one side when ldg-beta = +-1/2
        nsides = 0
        if kind == 'intcflux_ns':
            nsides = 1 if abs(m['tplargs']['c']['ldg-beta']) == 0.5 else 2
        # (the unit normal and its magnitude: nd + 1 values; with face
        # gradients in reference space an element column per side read,
        # whose metric terms are cache hits)
        vals = 4*nv + nd + 1 + nsides*nd*nv
        maps = 2 + 2*nsides + (nsides if m.get('facemet') else 0)
        return n*(vals*itemsize + maps*4)
    if kind == 'intconu':
        (n,) = m['dims']
        t = m['tplargs']
        nv, one = t['nvars'], abs(t['c']['ldg-beta']) == 0.5
        # One side read when ldg-beta = +-1/2 (else both); written to the
        # other side, or to both with both_sides (always both otherwise)
        nread = nv if one else 2*nv
        nwrite = 2*nv if (t.get('both_sides') or not one) else nv
        return n*((nread + nwrite)*itemsize + 4*4)
    if kind == 'negdivconf':
        nupts, neles = m['dims']
        nv = m['tplargs']['nvars']
        return (2*nv + 1)*nupts*neles*itemsize
    if kind == 'rkvdh2':
        r1 = m['r1']
        return 4*r1.nrow*r1.leaddim*itemsize
    if kind == 'rkmixed':
        # FP64 accumulator read + write, FP32 RHS read, FP32 input write
        return m['n']*(8 + 8 + 4 + 4)
    return 0


def kernel_flops64(k):
    """FP64 flops of one launch of an FP64 operator apply (the sparse
    kernel: one FMA per operator nonzero and column, plus one per output
    when it accumulates into the output)."""
    m = k.meta
    if k.name != 'mul':
        return 0
    ncol, nb = m['b'].ncol, m.get('nbatch', 1)
    nnz = 0
    for a in (m['a'], m.get('a2')):
        h = getattr(a, '_host', None) if a is not None else None
        if h is not None:
            nnz += int(np.count_nonzero(h))
    return nb*ncol*(2*nnz + (2*m['a'].nrow if m['beta'] else 0))


def fp64_peak(be):
    """Measured FP64 FMA throughput of the device, TFLOP/s."""
    import ctypes as C
    f = C.c_double()
    be.lib.probe_fp64_fma(1 << 14, C.byref(f), be.stream)
    return f.value/1e12


# Per-DoF HBM floor of one right-hand side (read the solution, write the
# RHS, vertices, face states and common fluxes; FP64, halved for FP32
# state) of the Navier-Stokes hex p=3 workload: 51 392 B per element of
# 320 DoF
FLOOR_BYTES_PER_DOF_F64 = 51392/320


def dram_traffic(form, kernel, n):
    """ncu DRAM bytes per launch of the dominant kernel, scaled from the
    committed capture (profiles/dram_traffic.json: bytes per column at the
    captured size) to n^3 elements; None without a capture."""
    p = ROOT / 'profiles' / 'dram_traffic.json'
    if not p.exists():
        return None
    d = json.loads(p.read_text()).get(form, {}).get(kernel)
    if not d:
        return None
    return int(d['bytes_per_element']*n**3)


def cpu_model():
    try:
        for line in Path('/proc/cpuinfo').read_text().splitlines():
            k, _, v = line.partition(':')
            if k.strip() in ('model name', 'Model'):
                return v.strip()
        out = subprocess.run(['lscpu'], capture_output=True, text=True,
                             timeout=10).stdout
        for line in out.splitlines():
            if line.startswith('Model name'):
                return line.split(':', 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    return None


def flat_kernels(klist):
    for k in klist:
        if hasattr(k, 'kernels'):
            yield from flat_kernels(k.kernels)
        else:
            yield k


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------

class Dist:
    def __init__(self, world):
        self.world = world

    def barrier(self):
        if self.world > 1:
            import torch.distributed as dist
            dist.barrier()

    def allmax(self, x):
        if self.world > 1:
            import torch
            import torch.distributed as dist
            t = torch.tensor([x], dtype=torch.float64)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            return float(t.item())
        return x


def make_form(form, args):
    from pyfr_gb300.backend import B200Backend
    from pyfr_gb300.cases import ns_tgv
    from pyfr_gb300.integrators import MixedRKIntegrator, RKVdH2Integrator
    from pyfr_gb300.solvers.system import NavierStokesSystem

    prec = 'double' if form == 'plain' else 'single'
    cfg, mesh = ns_tgv(n=args.n, order=3, dt=args.dt, precision=prec)
    cfg.set('backend-b200', 'device-id', str(args.local_rank))
    # The chosen form: split-BF16 data, the operator in three BF16 terms
    # where its image fits shared memory (five products, else four); the
    # three-product split is reported beside it
    if form in ('chosen', 'bf16x3'):
        cfg.set('backend-b200', 'mul-precision', 'bf16x3')
        cfg.set('backend-b200', 'split-products',
                str(args.chosen_products) if form == 'chosen' else '3')
    elif form == 'tf32':
        cfg.set('backend-b200', 'mul-precision', 'tf32')
    if not args.autotune:
        cfg.set('backend-b200', 'autotune', 'false')
    cfg.set('backend-b200', 'fuse-stage', args.fuse_stage)
    be = B200Backend(cfg)
    icls = RKVdH2Integrator if form == 'plain' else MixedRKIntegrator
    return icls(be, NavierStokesSystem, mesh, cfg)


def measure(intg, args, dist, e2e=True, profile=True):
    import ctypes as C

    be = intg.backend
    lib, stream = be.lib, be.stream

    def ev():
        e = C.c_void_p()
        lib.event_create(C.byref(e))
        return e.value

    def elapsed(a, b):
        ms = C.c_float()
        lib.event_elapsed(C.byref(ms), a, b)
        return ms.value

    def one_step():
        (idx,) = intg.step(intg.tcurr, intg.dt)[:1]
        intg.idxcurr = idx
        intg.tcurr += intg.dt

    # Warm-up (also captures the step graphs)
    for _ in range(args.warmup):
        one_step()
    be.wait()

    # Device-resident timed region
    e0, e1 = ev(), ev()
    dist.barrier()
    be.wait()
    with ClockSampler(args.local_rank) as clk:
        lib.event_record(e0, stream)
        for _ in range(args.steps):
            one_step()
        lib.event_record(e1, stream)
        lib.event_sync(e1)
    be.wait()
    dist.barrier()
    res = dict(t_ms=dist.allmax(elapsed(e0, e1)), clocks=clk.summary(),
               gndofs=intg.gndofs, nstages=intg.nstages,
               soln=intg.soln, nsteps=args.warmup + args.steps)

    klist, _ = intg.step_kernels(intg.idxcurr, intg.dt)
    klist = list(flat_kernels(klist))
    res['launches'] = len(klist)*args.steps

    if profile:
        # Per-kernel durations with events on the launching stream; the
        # replayed steps are undone afterwards so the solution history
        # stays in step with the other forms
        snap = intg.snapshot()
        per, ops = {}, {}
        evs = [ev() for _ in range(len(klist) + 1)]
        for _ in range(3):
            lib.event_record(evs[0], stream)
            for i, k in enumerate(klist):
                k.run(stream)
                lib.event_record(evs[i + 1], stream)
            lib.event_sync(evs[-1])
            for i, k in enumerate(klist):
                name = k.meta.get('kind', k.name)
                d = per.setdefault(name, {'ms': 0.0, 'n': 0, 'bytes': 0})
                t_ms, nb = elapsed(evs[i], evs[i + 1]), kernel_bytes(k, be)
                d['ms'] += t_ms
                d['n'] += 1
                d['bytes'] += nb
                if k.name == 'mul':
                    # Per operator apply: impl, shape(s), slices, beta
                    m = k.meta
                    key = f"{m.get('impl')} {m['a'].nrow}x{m['a'].ncol}"
                    if m.get('a2') is not None:
                        key += f"+{m['a2'].ncol}"
                    key += f" x{m.get('nbatch', 1)} beta={m['beta']:g}"
                    o = ops.setdefault(key, {'ms': 0.0, 'n': 0, 'bytes': 0})
                    o['ms'] += t_ms
                    o['n'] += 1
                    o['bytes'] += nb
        be.wait()
        intg.restore(snap)
        del snap
        tot = sum(d['ms'] for d in per.values())
        dom = max(per, key=lambda n: per[n]['ms'])
        d = per[dom]
        peak, peak_kind = _peaks()
        achieved = d['bytes']/(d['ms']*1e-3)/1e9
        # FP64 flops of the dominant kernel over the three replayed steps
        flops = 3*sum(kernel_flops64(k) for k in klist
                      if k.meta.get('kind', k.name) == dom)
        res['kernels'] = {
            n: {'share': round(v['ms']/tot, 4),
                'avg_us': round(1e3*v['ms']/v['n'], 2),
                'gbs': round(v['bytes']/(v['ms']*1e-3)/1e9, 1)}
            for n, v in sorted(per.items(), key=lambda x: -x[1]['ms'])}
        res['mul_ops'] = {
            n: {'avg_us': round(1e3*v['ms']/v['n'], 2),
                'gbs': round(v['bytes']/(v['ms']*1e-3)/1e9, 1)}
            for n, v in sorted(ops.items(), key=lambda x: -x[1]['ms'])}
        traffic = dram_traffic('plain' if be.fpdtype == np.float64
                               else 'chosen', dom, args.n)
        hbm = {'bound': 'hbm', 'kernel': dom, 'achieved': round(achieved, 1),
               'peak': peak, 'unit': 'GB/s', 'frac': round(achieved/peak, 4),
               'traffic': traffic, 'peak_source': f'{peak_kind} (HBM copy)',
               'alg_bytes_per_launch': int(d['bytes']/d['n']),
               'avg_launch_us': round(1e3*d['ms']/d['n'], 2)}
        if be.fpdtype == np.float64 and flops:
            # The FP64 sparse applies are bound by the FP64 pipe on this
            # GPU, not by HBM: report against the measured FMA throughput,
            # with the HBM fraction beside it
            pk = fp64_peak(be)
            tf = flops/(d['ms']*1e-3)/1e12
            res['roofline'] = {
                'bound': 'fp64', 'kernel': dom, 'achieved': round(tf, 4),
                'peak': round(pk, 4), 'unit': 'TFLOP/s',
                'frac': round(tf/pk, 4), 'traffic': traffic,
                'peak_source': 'measured (FP64 FMA-chain probe, '
                               'b200_probe_fp64_fma, this run)',
                'flops_per_launch': int(flops/d['n']),
                'avg_launch_us': round(1e3*d['ms']/d['n'], 2),
                'hbm': hbm}
        else:
            res['roofline'] = hbm

    if e2e:
        # End to end through the public API: the solution goes in from
        # pinned host memory and comes back every step.  Each step's result
        # makes a pipelined host round trip (b200_memcpy_roundtrip: down and
        # back up chunk by chunk, the two directions overlapping) into the
        # next step's input; the first input goes up whole and the last
        # result only comes down
        acc = hasattr(intg, 'acc')
        m = intg.acc[0] if acc else \
            intg.system.ele_banks[0][intg.idxcurr]
        nbytes = m.nbytes
        hbuf = C.c_void_p()
        lib.host_alloc(C.byref(hbuf), nbytes)
        lib.memcpy_dtoh(hbuf.value, m.data, nbytes, stream)
        be.wait()
        dist.barrier()
        lib.event_record(e0, stream)
        lib.memcpy_htod(m.data, hbuf.value, nbytes, stream)
        for i in range(args.steps):
            if acc:
                intg.refresh_input(stream)
            one_step()
            if not acc:
                # The result is the next step's input register
                m = intg.system.ele_banks[0][intg.idxcurr]
            last = i == args.steps - 1
            lib.memcpy_roundtrip(hbuf.value, m.data, None if last else m.data,
                                 nbytes, args.e2e_chunks, args.e2e_streams,
                                 stream)
        lib.event_record(e1, stream)
        lib.event_sync(e1)
        dist.barrier()
        res['te2e_ms'] = dist.allmax(elapsed(e0, e1))
        res['e2e_bytes'] = nbytes
        lib.host_free(hbuf.value)

    return res


def history(intg, nsteps, every):
    """Advance to step ``nsteps`` (counted from the initial condition),
    logging the normalised kinetic energy E_k = int rho|u|^2/(2 V) every
    ``every`` steps; returns the final solution and the E_k history."""
    from pyfr_gb300.plugins import FieldIntegrals

    fi = FieldIntegrals(intg)
    hist = {}
    while intg.nsteps < nsteps:
        k = min(every - intg.nsteps % every, nsteps - intg.nsteps)
        intg.run_steps(k)
        if intg.nsteps % every == 0:
            r = fi()
            hist[intg.nsteps] = 0.5*r['E']/r['vol']
    if intg.nsteps not in hist:
        r = fi()
        hist[intg.nsteps] = 0.5*r['E']/r['vol']
    return intg.soln, hist


def run_gpu(args, dist):
    import __graft_entry__ as ge
    ge.build_library()

    import numpy as np

    plain = make_form('plain', args)
    rp = measure(plain, args, dist)
    rp['neles'] = args.n**3
    (up,), hp = history(plain, args.accuracy_steps, args.ke_every)
    del plain

    out = {'plain': rp}
    forms = ['chosen', 'bf16x3', 'tf32', 'fp32'] if args.chosen else []
    for form in forms:
        intg = make_form(form, args)
        rc = measure(intg, args, dist)
        # Same initial condition and dt, advanced to the same step:
        # relative L2 error and kinetic-energy history error vs FP64
        (uc,), hc = history(intg, args.accuracy_steps, args.ke_every)
        rc['l2_err'] = float(np.linalg.norm((uc - up).ravel()) /
                             np.linalg.norm(up.ravel()))
        common = [s for s in hp if s in hc]
        rc['ke_err'] = float(max(abs(hc[s] - hp[s]) for s in common))
        rc['ke_final'] = hc[max(hc)]
        out[form] = rc
        del intg
    out['plain']['ke_final'] = hp[max(hp)]
    return out


def run_large(args, dist):
    """The large configuration: the chosen form on an n^3 TGV (memory model
    large, 64-bit gather maps) under the PI controller (rtol = atol =
    1e-6, error norm reduced in FP64) for a number of accepted steps, and
    the plain FP64 form on a smaller mesh with fixed steps for comparison.
    GDoF/s counts every RHS evaluation, rejected attempts included."""
    import ctypes as C

    import __graft_entry__ as ge
    from pyfr_gb300.backend import B200Backend
    from pyfr_gb300.cases import ns_tgv
    from pyfr_gb300.integrators import MixedRKIntegrator, RKVdH2Integrator
    from pyfr_gb300.solvers.system import NavierStokesSystem
    ge.build_library()

    def timed(intg, fn):
        lib, stream = intg.backend.lib, intg.backend.stream
        ev = [C.c_void_p(), C.c_void_p()]
        for e in ev:
            lib.event_create(C.byref(e))
        intg.backend.wait()
        dist.barrier()
        with ClockSampler(args.local_rank) as clk:
            lib.event_record(ev[0].value, stream)
            out = fn()
            lib.event_record(ev[1].value, stream)
            lib.event_sync(ev[1].value)
        ms = C.c_float()
        lib.event_elapsed(C.byref(ms), ev[0].value, ev[1].value)
        return out, dist.allmax(ms.value), clk.summary()

    res = {}
    t0 = time.perf_counter()
    cfg, mesh = ns_tgv(n=args.large_n, order=3, dt=args.dt, precision='single',
                       memory_model='large')
    cfg.set('backend-b200', 'device-id', str(args.local_rank))
    cfg.set('backend-b200', 'mul-precision', 'bf16x3')
    cfg.set('backend-b200', 'split-products', str(args.chosen_products))
    sect = 'solver-time-integrator'
    cfg.set(sect, 'controller', 'pi')
    cfg.set(sect, 'rtol', '1e-6')
    cfg.set(sect, 'atol', '1e-6')
    intg = MixedRKIntegrator(B200Backend(cfg), NavierStokesSystem, mesh, cfg)
    setup_s = time.perf_counter() - t0
    intg.run_pi_steps(2)                  # warm-up (graph captures)
    n0, r0 = intg.nacptsteps, intg.nrjctsteps
    attempts, ms, clk = timed(intg, lambda: intg.run_pi_steps(args.large_steps))
    nrhs = attempts*intg.nstages
    # The same integrator stepping at a fixed dt (the controller's error
    # norm and host round trip left out), for the cost of adaptivity
    _, ms_fixed, _ = timed(intg, lambda: intg.run_steps(args.large_steps,
                                                         intg.dt))
    be = intg.backend
    res['chosen'] = {
        'neles': args.large_n**3, 'ndofs': intg.gndofs,
        'accepted_steps': intg.nacptsteps - n0,
        'rejected_steps': intg.nrjctsteps - r0,
        'dt_final': intg.dt, 't_final': intg.tcurr,
        'ms': ms, 'gdofs': dist.world*intg.gndofs*nrhs/(ms*1e-3)/1e9,
        'fixed_dt_gdofs': dist.world*intg.gndofs*args.large_steps *
        intg.nstages/(ms_fixed*1e-3)/1e9,
        'device_gb': be.memory_info().peak/1e9, 'setup_s': setup_s,
        'clocks': clk}
    del intg, be

    t0 = time.perf_counter()
    cfg, mesh = ns_tgv(n=args.large_plain_n, order=3, dt=args.dt,
                       precision='double', memory_model='large')
    cfg.set('backend-b200', 'device-id', str(args.local_rank))
    intg = RKVdH2Integrator(B200Backend(cfg), NavierStokesSystem, mesh, cfg)
    setup_s = time.perf_counter() - t0
    intg.run_steps(1)
    _, ms, clk = timed(intg, lambda: intg.run_steps(args.large_plain_steps))
    nrhs = args.large_plain_steps*intg.nstages
    res['plain'] = {
        'neles': args.large_plain_n**3, 'ndofs': intg.gndofs,
        'steps': args.large_plain_steps, 'ms': ms,
        'gdofs': dist.world*intg.gndofs*nrhs/(ms*1e-3)/1e9,
        'device_gb': intg.backend.memory_info().peak/1e9, 'setup_s': setup_s,
        'clocks': clk}
    return res


def run_ensemble(args, dist, unbatched=True):
    """The batching configuration's ensemble: independent 2-D vortex cases
    of uneven size (quads per side uniform in 16..96), order (2, 3, 4) and
    strength (beta uniform in 2..6) from one seed, merged by order and
    advanced in one CUDA graph per step; plain FP64 and the chosen form,
    and for comparison the same cases advanced one system each."""
    import ctypes as C

    import __graft_entry__ as ge
    from pyfr_gb300.backend import B200Backend
    from pyfr_gb300.cases import euler_vortex
    from pyfr_gb300.ensemble import Ensemble, vortex_cases
    from pyfr_gb300.inifile import Inifile
    from pyfr_gb300.integrators import RKVdH2Integrator
    from pyfr_gb300.solvers.system import EulerSystem
    ge.build_library()

    def backend(prec, mul='native'):
        cfg = Inifile()
        cfg.set('backend', 'precision', prec)
        cfg.set('backend-b200', 'device-id', str(args.local_rank))
        cfg.set('backend-b200', 'mul-precision', mul)
        cfg.set('backend-b200', 'split-products', str(args.chosen_products))
        return B200Backend(cfg)

    def timed(be, fn):
        lib, stream = be.lib, be.stream
        ev = [C.c_void_p(), C.c_void_p()]
        for e in ev:
            lib.event_create(C.byref(e))
        be.wait()
        dist.barrier()
        with ClockSampler(args.local_rank) as clk:
            lib.event_record(ev[0].value, stream)
            fn()
            lib.event_record(ev[1].value, stream)
            lib.event_sync(ev[1].value)
        ms = C.c_float()
        lib.event_elapsed(C.byref(ms), ev[0].value, ev[1].value)
        return dist.allmax(ms.value), clk.summary()

    cases = vortex_cases(args.ens_cases, seed=args.ens_seed)
    nsteps, dt = args.steps, args.ens_dt
    res = {'ncases': len(cases), 'seed': args.ens_seed, 'dt': dt,
           'orders': {p: sum(c['order'] == p for c in cases)
                      for p in (2, 3, 4)}}
    ens = {}
    for form, prec, mul in [('plain', 'double', 'native'),
                            ('chosen', 'single', 'bf16x3')]:
        be = backend(prec, mul)
        e = Ensemble(be, cases, dt, prec, mixed=form == 'chosen')
        e.run_steps(args.warmup)
        ms, clk = timed(be, lambda: e.run_steps(nsteps))
        gd = dist.world*e.gndofs*e.nstages*nsteps/(ms*1e-3)/1e9
        res[form] = {'gdofs': gd, 'ms_per_step': ms/nsteps, 'clocks': clk,
                     'ndofs': e.gndofs, 'systems': len(e.intgs)}
        ens[form] = e

    # Per-case L2 error of the chosen form against plain FP64
    up, uc = ens['plain'].case_solutions(), ens['chosen'].case_solutions()
    res['chosen']['l2_err_vs_fp64_max'] = max(
        float(np.linalg.norm(uc[k] - up[k])/np.linalg.norm(up[k]))
        for k in up)
    res['chosen']['accuracy_after_steps'] = args.warmup + nsteps
    del ens

    if not unbatched:
        return res

    # The same cases one system each (plain FP64), for the batching gain
    be = backend('double')
    intgs = []
    for c in cases:
        cfg, mesh = euler_vortex(n=c['n'], order=c['order'], dt=dt,
                                 beta=c['beta'])
        intgs.append(RKVdH2Integrator(be, EulerSystem, mesh, cfg))
    for i in intgs:
        i.run_steps(args.warmup)

    def one_by_one():
        for _ in range(nsteps):
            for i in intgs:
                (i.idxcurr,) = i.step(i.tcurr, dt)[:1]
                i.tcurr += dt
        be.wait()
    ms, clk = timed(be, one_by_one)
    nd = sum(i.gndofs for i in intgs)
    res['plain_unbatched'] = {'gdofs': dist.world*nd*5*nsteps/(ms*1e-3)/1e9,
                              'ms_per_step': ms/nsteps, 'systems': len(intgs)}
    return res


def run_mixed(args, dist, forms=('plain', 'chosen', 'tf32')):
    """The batching configuration's mixed meshes: 3-D Euler on a periodic
    box of n^3 cells, hexahedra and prisms, prisms and tetrahedra, or
    hexahedra and tetrahedra joined by pyramids (p = 3; an advected
    density wave), plain FP64 and the chosen form; one CUDA graph per RK45
    step over every element type."""
    import ctypes as C

    import __graft_entry__ as ge
    from pyfr_gb300.backend import B200Backend
    from pyfr_gb300.cases import euler_mixed
    from pyfr_gb300.integrators import MixedRKIntegrator, RKVdH2Integrator
    from pyfr_gb300.solvers.system import EulerSystem
    ge.build_library()

    def timed(be, fn):
        lib, stream = be.lib, be.stream
        ev = [C.c_void_p(), C.c_void_p()]
        for e in ev:
            lib.event_create(C.byref(e))
        be.wait()
        dist.barrier()
        with ClockSampler(args.local_rank) as clk:
            lib.event_record(ev[0].value, stream)
            fn()
            lib.event_record(ev[1].value, stream)
            lib.event_sync(ev[1].value)
        ms = C.c_float()
        lib.event_elapsed(C.byref(ms), ev[0].value, ev[1].value)
        return dist.allmax(ms.value), clk.summary()

    res = {}
    for kinds in args.mixed_kinds.split(','):
        out, solns = {}, {}
        for form in forms:
            prec = 'double' if form == 'plain' else 'single'
            cfg, mesh = euler_mixed(n=args.mixed_n, order=args.mixed_order,
                                    kinds=kinds, dt=args.mixed_dt,
                                    precision=prec)
            cfg.set('backend-b200', 'device-id', str(args.local_rank))
            icls = RKVdH2Integrator
            if form == 'chosen':
                cfg.set('backend-b200', 'mul-precision', 'bf16x3')
                cfg.set('backend-b200', 'split-products',
                        str(args.chosen_products))
                icls = MixedRKIntegrator
            elif form == 'tf32':
                cfg.set('backend-b200', 'mul-precision', 'tf32')
                icls = MixedRKIntegrator
            be = B200Backend(cfg)
            intg = icls(be, EulerSystem, mesh, cfg)
            intg.run_steps(args.warmup)
            ms, clk = timed(be, lambda: intg.run_steps(args.steps))
            nrhs = args.steps*intg.nstages
            out[form] = {
                'gdofs': dist.world*intg.gndofs*nrhs/(ms*1e-3)/1e9,
                'ms_per_step': ms/args.steps, 'clocks': clk,
                'ndofs': intg.gndofs,
                'neles': {et: int(v.shape[1]) for et, v in mesh.spts.items()}}
            solns[form] = [np.asarray(u, dtype=np.float64)
                           for u in intg.soln]
            del intg, be
        for form in forms[1:]:
            out[form]['l2_err_vs_fp64'] = max(
                float(np.linalg.norm(a - b)/np.linalg.norm(b))
                for a, b in zip(solns[form], solns['plain']))
            out[form]['accuracy_after_steps'] = args.warmup + args.steps
            out[f'speedup_{form}_vs_plain'] = \
                out[form]['gdofs']/out['plain']['gdofs']
        res[kinds] = out
    return res


def run_batching(args, dist):
    """The batching configuration in the default run, compactly: the
    32^3-cell box where hexahedra meet tetrahedra through pyramids (3-D
    Euler density wave, p = 3) and the 64-case vortex ensemble, each in
    plain FP64 and the chosen form, 20 timed RK45 steps after 3 warm-up
    steps, with the chosen form's L2 error against plain FP64."""
    a = argparse.Namespace(**vars(args))
    a.steps, a.warmup = 20, 3
    a.mixed_kinds = 'hex-pyr-tet'
    m = run_mixed(a, dist, forms=('plain', 'chosen'))['hex-pyr-tet']
    e = run_ensemble(a, dist, unbatched=False)

    def short(r, f):
        d = {'gdofs': round(r[f]['gdofs'], 3),
             'ms_per_step': round(r[f]['ms_per_step'], 3)}
        for k in ('l2_err_vs_fp64', 'l2_err_vs_fp64_max'):
            if k in r[f]:
                d[k] = r[f][k]
        return d

    return {
        'mixed_hex_pyr_tet': {
            'config': f'{args.mixed_n}^3 cells: '
                      + ', '.join(f'{n} {k}' for k, n in
                                  m['plain']['neles'].items())
                      + f', p=3, {m["plain"]["ndofs"]} DoF',
            'plain': short(m, 'plain'), 'chosen': short(m, 'chosen'),
            'speedup': round(m['speedup_chosen_vs_plain'], 2)},
        'ensemble': {
            'config': f'{e["ncases"]} 2-D vortex cases, p in 2-4, '
                      f'{e["plain"]["ndofs"]} DoF, {e["plain"]["systems"]} '
                      'systems in one graph per step',
            'plain': short(e, 'plain'), 'chosen': short(e, 'chosen'),
            'speedup': round(e['chosen']['gdofs']/e['plain']['gdofs'], 2)},
        'steps': a.steps, 'warmup': a.warmup}


# ---------------------------------------------------------------------------
# CPU arm (the oracle restatement, bounded sample)
# ---------------------------------------------------------------------------

def run_cpu_sample(n_sample, seconds=10.0):
    """Time the C/OpenMP oracle's RHS (compiled with the reference OpenMP
    backend's -O3 -ffast-math, all host cores) on an n_sample^3 TGV mesh,
    repeating RHS evaluations for about ``seconds``."""
    from oracle.c_oracle import COracle
    from pyfr_gb300.cases import ns_tgv
    from pyfr_gb300.solvers.elements import NavierStokesElements
    from tests.oracle_util import disc_for_mesh

    cfg, mesh = ns_tgv(n=n_sample, order=3)
    e = NavierStokesElements('hex', mesh.spts['hex'], cfg)
    u = e.set_ics_from_cfg()
    d = disc_for_mesh(mesh, 3, ns=True)
    c = cfg.items_as('constants', float) | cfg.items_as('solver-interfaces',
                                                       float)
    co = COracle(d, c, variant='fast')
    ue = np.ascontiguousarray(u.transpose(2, 0, 1))
    co.rhs_native(ue)

    nrhs, t0 = 0, time.perf_counter()
    while (dt := time.perf_counter() - t0) < seconds or nrhs < 2:
        co.rhs_native(ue)
        nrhs += 1
    ndofs = u.size
    return ndofs*nrhs/dt/1e9, dt, ndofs, nrhs


def cpu_cores():
    return int(os.environ.get('OMP_NUM_THREADS', os.cpu_count() or 1))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=20)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='b200', choices=['b200', 'reference'])
    ap.add_argument('--n', type=int, default=48)
    ap.add_argument('--dt', type=float, default=5e-4)
    ap.add_argument('--cpu-sample', type=int, default=None,
                    help='mesh size n^3 of the CPU timing (default: --n, '
                         'the benchmark mesh itself)')
    ap.add_argument('--cpu-seconds', type=float, default=10.0)
    ap.add_argument('--no-chosen', dest='chosen', action='store_false',
                    help='skip the chosen precision form')
    ap.add_argument('--chosen-products', type=int, default=5, choices=[3, 4, 5],
                    help='split-BF16 products of the chosen form')
    ap.add_argument('--accuracy-steps', type=int, default=200,
                    help='steps after which the chosen form is compared '
                         'with FP64')
    ap.add_argument('--ke-every', type=int, default=10)
    ap.add_argument('--large', action='store_true',
                    help='the large configuration (chosen form at '
                         '--large-n^3 under the PI controller, plain FP64 at '
                         '--large-plain-n^3) instead of the headline run')
    ap.add_argument('--large-n', type=int, default=128)
    ap.add_argument('--large-steps', type=int, default=100)
    ap.add_argument('--large-plain-n', type=int, default=96)
    ap.add_argument('--large-plain-steps', type=int, default=5)
    ap.add_argument('--mixed', action='store_true',
                    help='time the mixed meshes (hexahedra/prisms, '
                    'prisms/tetrahedra, hexahedra/pyramids/tetrahedra) '
                    'instead')
    ap.add_argument('--mixed-n', type=int, default=32)
    ap.add_argument('--mixed-order', type=int, default=3)
    ap.add_argument('--mixed-dt', type=float, default=1e-3)
    ap.add_argument('--mixed-kinds', default='hex-pri,pri-tet,hex-pyr-tet',
                    help='comma-separated mixed meshes for --mixed')
    ap.add_argument('--e2e-chunks', type=int, default=16,
                    help='pieces of the pipelined host round trip of the '
                         'end-to-end loop')
    ap.add_argument('--e2e-streams', type=int, default=2,
                    help='copy streams per direction of the round trip')
    ap.add_argument('--no-batching', dest='batching', action='store_false',
                    help='leave out the batching summary of the default run '
                         '(the hexahedron-pyramid-tetrahedron box and the '
                         'vortex ensemble, plain FP64 and chosen form)')
    ap.add_argument('--ensemble', action='store_true',
                    help='the batching configuration\'s ensemble of 2-D '
                         'vortex cases instead of the headline run')
    ap.add_argument('--ens-cases', type=int, default=64)
    ap.add_argument('--ens-seed', type=int, default=0)
    ap.add_argument('--ens-dt', type=float, default=1e-4)
    ap.add_argument('--fuse-stage', default='auto',
                    choices=['auto', 'true', 'false'],
                    help='the RK stage in the divergence apply\'s epilogue '
                         '(chosen form)')
    ap.add_argument('--no-autotune', dest='autotune', action='store_false',
                    help='the deepest pipeline plan of each operator instead '
                         'of timing them (no tuning launches before the '
                         'timed ones: a fixed launch sequence to profile)')
    ap.add_argument('--only', choices=['plain', 'chosen', 'bf16x3', 'tf32',
                                       'fp32'],
                    help='time one precision form alone (no accuracy '
                         'history, end-to-end loop or CPU sample): the '
                         'command to run under a profiler')
    args = ap.parse_args()
    if args.cpu_sample is None:
        args.cpu_sample = args.n

    world = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    args.local_rank = int(os.environ.get('LOCAL_RANK', '0'))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group('gloo')

    workload = {'workload': f'3-D Navier-Stokes Taylor-Green vortex, {args.n}^3 '
                            'hex, p=3 Gauss-Legendre, Rusanov+LDG, RK45, '
                            'plain FP64',
                'neles': args.n**3, 'order': 3,
                'l2': 'inputs larger than L2 (state 283 MB per register)'}

    if args.impl == 'reference':
        if rank != 0:
            return
        os.environ.setdefault('OMP_NUM_THREADS', str(os.cpu_count() or 1))
        secs = min(max(2.0, 2.0*args.steps), 60.0)
        v, dt, ndofs, nrhs = run_cpu_sample(args.cpu_sample, secs)
        sample = (f'{args.cpu_sample}^3-element TGV ({ndofs} DoF), {nrhs} '
                  f'RHS evaluations in {dt:.1f} s, C/OpenMP restatement of '
                  'the reference kernels (-O3 -ffast-math, the reference '
                  'OpenMP backend\'s flags)')
        print(json.dumps({
            'impl': 'reference', 'metric': METRIC, 'value': v,
            'unit': 'GDoF/s', 'n_gpus': args.gpus, 'steps': args.steps,
            'warmup': args.warmup, 'higher_is_better': True,
            'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64',
            'data': 'synthetic', 'config': workload,
            'same_mesh': args.cpu_sample == args.n,
            'cpu_baseline': {'value': v, 'unit': 'GDoF/s',
                             'cores': cpu_cores(), 'kind': 'port',
                             'cpu_model': cpu_model(), 'sample': sample},
            'e2e': {'value': v, 'unit': 'GDoF/s', 'h2d_bytes_per_step': 0,
                    'd2h_bytes_per_step': 0}}))
        return

    if args.ensemble:
        r = run_ensemble(args, Dist(world))
        if rank == 0:
            print(json.dumps({
                'metric': METRIC, 'unit': 'GDoF/s', 'n_gpus': world,
                'steps': args.steps, 'warmup': args.warmup,
                'config': {'workload': '2-D Euler isentropic-vortex '
                                       'ensemble, merged by order, one CUDA '
                                       'graph per RK45 step'},
                'data': 'synthetic'} | r))
        return

    if args.mixed:
        r = run_mixed(args, Dist(world))
        if rank == 0:
            print(json.dumps({
                'metric': METRIC, 'unit': 'GDoF/s', 'n_gpus': world,
                'steps': args.steps, 'warmup': args.warmup,
                'config': {'workload': f'3-D Euler, periodic '
                                       f'{args.mixed_n}^3-cell boxes '
                                       f'({args.mixed_kinds}), '
                                       f'p={args.mixed_order}, density '
                                       'wave, one CUDA graph per RK45 step',
                           'dt': args.mixed_dt},
                'data': 'synthetic'} | r))
        return

    if args.large:
        r = run_large(args, Dist(world))
        if rank == 0:
            print(json.dumps({
                'metric': METRIC, 'unit': 'GDoF/s', 'n_gpus': world,
                'config': {
                    'workload': f'3-D Navier-Stokes Taylor-Green vortex, '
                                f'{args.large_n}^3 hex, p=3, chosen form, '
                                'RK45 with the PI controller (rtol = atol = '
                                '1e-6, FP64 error norm), memory-model large; '
                                f'plain FP64 at {args.large_plain_n}^3',
                    'accepted_steps': args.large_steps},
                'data': 'synthetic', 'chosen': r['chosen'],
                'plain': r['plain'],
                'speedup_vs_plain': r['chosen']['gdofs']/r['plain']['gdofs'],
                'host_maxrss_gb': resource.getrusage(
                    resource.RUSAGE_SELF).ru_maxrss/2**20}))
        return

    if args.only:
        import __graft_entry__ as ge
        ge.build_library()
        intg = make_form(args.only, args)
        r = measure(intg, args, Dist(world), e2e=False, profile=False)
        if rank == 0:
            print(json.dumps({
                'form': args.only, 'n': args.n, 'steps': args.steps,
                'ms_per_step': r['t_ms']/args.steps,
                'gdofs': world*r['gndofs']*r['nstages']*args.steps /
                (r['t_ms']*1e-3)/1e9}))
        return

    allres = run_gpu(args, Dist(world))
    batching = run_batching(args, Dist(world)) if args.batching else None
    if rank != 0:
        return

    def gdofs(r, key='t_ms'):
        return world*r['gndofs']*r['nstages']*args.steps/(r[key]*1e-3)/1e9

    res = allres['plain']
    value, e2e = gdofs(res), gdofs(res, 'te2e_ms')
    finite = bool(all(np.isfinite(u).all() for u in res['soln']))

    os.environ.setdefault('OMP_NUM_THREADS', str(os.cpu_count() or 1))
    cpu_v, cpu_dt, cpu_ndofs, cpu_nrhs = run_cpu_sample(args.cpu_sample,
                                                        args.cpu_seconds)

    chosen = None
    labels = {
        'chosen': f'operator contractions split-BF16 (data hi/lo, operator '
                  f'in {3 if args.chosen_products == 5 else 2} terms where it '
                  f'fits), {args.chosen_products} products, on tcgen05 '
                  'tensor cores '
                  '(FP32 accumulate, fused applies), FP32 fluxes on the '
                  'reference-state transform, FP64 RK accumulation',
        'bf16x3': 'operator contractions split-BF16 hi/lo, 3 products '
                  '(Ahi*Bhi + Ahi*Blo + Alo*Bhi) on tcgen05 tensor cores, '
                  'otherwise as chosen',
        'tf32': 'operator contractions TF32 (one product) on tcgen05 '
                'tensor cores, otherwise as chosen',
        'fp32': 'operator contractions FP32 (sparse, CUDA cores), FP32 '
                'fluxes, FP64 RK accumulation'}
    variants = {}
    for form in ('chosen', 'bf16x3', 'tf32', 'fp32'):
        if form not in allres:
            continue
        rc = allres[form]
        variants[form] = {
            'form': labels[form],
            'value': gdofs(rc), 'unit': 'GDoF/s',
            'ms_per_step': rc['t_ms']/args.steps,
            'l2_err_vs_fp64': rc['l2_err'],
            'ke_hist_max_abs_err_vs_fp64': rc['ke_err'],
            'accuracy_after_steps': args.accuracy_steps,
            'speedup_vs_plain': gdofs(rc)/value,
            'clocks': rc['clocks'], 'gpu_launches': rc['launches']}
        if 'te2e_ms' in rc:
            variants[form]['e2e'] = {
                'value': gdofs(rc, 'te2e_ms'), 'unit': 'GDoF/s',
                'h2d_bytes_per_step': rc['e2e_bytes'],
                'd2h_bytes_per_step': rc['e2e_bytes']}
        if 'roofline' in rc:
            variants[form] |= {'roofline': rc['roofline'],
                               'kernels': rc['kernels'],
                               'mul_ops': rc['mul_ops']}
    chosen = variants.pop('chosen', None)
    if chosen is not None:
        chosen['other_variants'] = variants

    # Step-level fraction of the HBM floor: the algorithmic floor bytes of
    # every right-hand side of the timed steps over the time, against the
    # measured copy bandwidth
    peak, _ = _peaks()

    def floor_frac(r, itemsize):
        b = FLOOR_BYTES_PER_DOF_F64*itemsize/8*r['gndofs']*r['nstages']
        return round(b*args.steps/(r['t_ms']*1e-3)/1e9/peak, 4)

    out = {
        'metric': METRIC, 'value': value, 'unit': 'GDoF/s',
        'n_gpus': world, 'steps': args.steps, 'warmup': args.warmup,
        'ms_per_step': res['t_ms']/args.steps, 'higher_is_better': True,
        'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64',
        'data': 'synthetic', 'config': workload | {
            'ndofs': res['gndofs'], 'dt': args.dt,
            'parallelism': 'replicas' if world > 1 else 'single-gpu'},
        'finite': finite,
        'clocks': res['clocks'],
        'e2e': {'value': e2e, 'unit': 'GDoF/s',
                'h2d_bytes_per_step': res['e2e_bytes'],
                'd2h_bytes_per_step': res['e2e_bytes']},
        'gpu_launches': res['launches'],
        'roofline': res['roofline'],
        'kernels': res['kernels'],
        'mul_ops': res['mul_ops'],
        'chosen': chosen,
        'floor_frac': floor_frac(res, 8),
        'cpu_baseline': {'value': cpu_v, 'unit': 'GDoF/s',
                         'cores': cpu_cores(), 'kind': 'port',
                         'cpu_model': cpu_model(),
                         'same_mesh': args.cpu_sample == args.n,
                         'sample': f'{cpu_nrhs} RHS evaluations of the '
                                   f'C/OpenMP oracle (-O3 -ffast-math) on a '
                                   f'{args.cpu_sample}^3 TGV mesh '
                                   f'({cpu_ndofs} DoF, {cpu_dt:.1f} s)'},
    }
    if batching is not None:
        out['batching_summary'] = batching
    if chosen is not None:
        rc = allres['chosen']
        chosen['floor_frac'] = floor_frac(rc, 4)
        # A compact summary of the chosen form last, so that a reader of a
        # truncated line still sees it
        out['chosen_summary'] = {
            'value': round(chosen['value'], 3), 'unit': 'GDoF/s',
            'ms_per_step': round(chosen['ms_per_step'], 3),
            'speedup_vs_plain': round(chosen['speedup_vs_plain'], 2),
            'l2_err_vs_fp64': chosen['l2_err_vs_fp64'],
            'ke_hist_max_abs_err_vs_fp64':
                chosen['ke_hist_max_abs_err_vs_fp64'],
            'after_steps': args.accuracy_steps,
            'roofline_frac': chosen.get('roofline', {}).get('frac'),
            'floor_frac': chosen['floor_frac'],
            'e2e': round(chosen['e2e']['value'], 3) if 'e2e' in chosen
            else None}
    print(json.dumps(out))


if __name__ == '__main__':
    main()
