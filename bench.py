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
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

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

def kernel_bytes(k, itemsize):
    m = k.meta
    kind = m.get('kind', k.name)
    if k.name == 'mul':
        a, b, out = m['a'], m['b'], m['out']
        ncol = b.ncol
        nout = a.nrow*ncol*(2 if m['beta'] else 1)
        return (a.ncol*ncol + nout)*itemsize
    if kind in ('tflux_ns', 'tflux_euler'):
        nupts, neles = m['dims']
        nd, nv = m['tplargs']['ndims'], m['tplargs']['nvars']
        per_pt = nv + nd*nv + (2*nd*nv if kind == 'tflux_ns' else 0)
        geo = (2**nd)*nd*neles if m.get('verts') is not None else \
            nupts*neles*(nd*nd + 1)
        return (per_pt*nupts*neles + geo)*itemsize
    if kind in ('intcflux_ns', 'intcflux_euler'):
        (n,) = m['dims']
        nd, nv = m['tplargs']['ndims'], m['tplargs']['nvars']
        vals = 4*nv + nd + (2*nd*nv if kind == 'intcflux_ns' else 0)
        maps = 2 + (4 if kind == 'intcflux_ns' else 0)
        return n*(vals*itemsize + maps*4)
    if kind == 'intconu':
        (n,) = m['dims']
        nv = m['tplargs']['nvars']
        return n*(2*nv*itemsize + 4*4)
    if kind == 'negdivconf':
        nupts, neles = m['dims']
        nv = m['tplargs']['nvars']
        return (2*nv + 1)*nupts*neles*itemsize
    if kind == 'rkvdh2':
        r1 = m['r1']
        return 4*r1.nrow*r1.leaddim*itemsize
    return 0


def flat_kernels(klist):
    for k in klist:
        if hasattr(k, 'kernels'):
            yield from flat_kernels(k.kernels)
        else:
            yield k


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------

def run_gpu(args, rank, world):
    import ctypes as C

    import numpy as np

    import __graft_entry__ as ge
    ge.build_library()

    from pyfr_gb300.backend import B200Backend
    from pyfr_gb300.cases import ns_tgv
    from pyfr_gb300.integrators import RKVdH2Integrator
    from pyfr_gb300.solvers.system import NavierStokesSystem

    cfg, mesh = ns_tgv(n=args.n, order=3, dt=args.dt)
    cfg.set('backend-b200', 'device-id', str(args.local_rank))
    be = B200Backend(cfg)
    lib, stream = be.lib, be.stream
    intg = RKVdH2Integrator(be, NavierStokesSystem, mesh, cfg)
    gndofs = intg.gndofs
    nstages = intg.nstages
    itemsize = 8

    def ev():
        e = C.c_void_p()
        lib.event_create(C.byref(e))
        return e.value

    def elapsed(a, b):
        ms = C.c_float()
        lib.event_elapsed(C.byref(ms), a, b)
        return ms.value

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    def allmax(x):
        if world > 1:
            import torch
            import torch.distributed as dist
            t = torch.tensor([x], dtype=torch.float64)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            return float(t.item())
        return x

    # Warm-up (also captures the step graphs)
    for _ in range(args.warmup):
        intg.run_steps(1)
    be.wait()

    # Device-resident timed region
    e0, e1 = ev(), ev()
    barrier()
    be.wait()
    with ClockSampler(args.local_rank) as clk:
        lib.event_record(e0, stream)
        for _ in range(args.steps):
            (idx,) = intg.step(intg.tcurr, intg.dt)[:1]
            intg.idxcurr = idx
            intg.tcurr += intg.dt
        lib.event_record(e1, stream)
        lib.event_sync(e1)
    be.wait()
    barrier()
    t_ms = allmax(elapsed(e0, e1))

    (u,) = intg.soln
    finite = bool(np.isfinite(u).all())

    # Kernel launches per step
    klist = []
    r1, r2, rs = intg._regs(intg.idxcurr)
    for i in range(nstages):
        for g in intg.system.rhs_graphs(r2 if i else r1, r2):
            klist.extend(flat_kernels(g.klist))
        klist.extend(intg._rk_kerns(i, r1, r2, *rs))
        r1, r2 = r2, r1
    launches_per_step = len(klist)

    # Per-kernel durations with events on the launching stream
    per = {}
    nrep = 3
    evs = [ev() for _ in range(len(klist) + 1)]
    for _ in range(nrep):
        lib.event_record(evs[0], stream)
        for i, k in enumerate(klist):
            if hasattr(k, 'rtargs'):
                k.bind(dt=intg.dt)
            k.run(stream)
            lib.event_record(evs[i + 1], stream)
        lib.event_sync(evs[-1])
        for i, k in enumerate(klist):
            name = k.meta.get('kind', k.name)
            d = per.setdefault(name, {'ms': 0.0, 'n': 0, 'bytes': 0})
            d['ms'] += elapsed(evs[i], evs[i + 1])
            d['n'] += 1
            d['bytes'] += kernel_bytes(k, itemsize)
    be.wait()
    tot = sum(d['ms'] for d in per.values())
    dom = max(per, key=lambda n: per[n]['ms'])
    d = per[dom]
    peak, peak_kind = _peaks()
    achieved = d['bytes']/(d['ms']*1e-3)/1e9
    kernels = {n: {'share': round(v['ms']/tot, 4),
                   'avg_us': round(1e3*v['ms']/v['n'], 2),
                   'gbs': round(v['bytes']/(v['ms']*1e-3)/1e9, 1)}
               for n, v in sorted(per.items(), key=lambda x: -x[1]['ms'])}

    # End-to-end through the public API: pinned host solution in, one step,
    # solution out, every step
    bank = intg.system.ele_banks[0]
    nbytes = bank[0].nbytes
    hbuf = C.c_void_p()
    lib.host_alloc(C.byref(hbuf), nbytes)
    lib.memcpy_dtoh(hbuf.value, bank[intg.idxcurr].data, nbytes, stream)
    be.wait()
    for _ in range(2):
        intg.run_steps(1)
    be.wait()
    barrier()
    t0 = time.perf_counter()
    lib.event_record(e0, stream)
    for _ in range(args.steps):
        lib.memcpy_htod(bank[intg.idxcurr].data, hbuf.value, nbytes, stream)
        (idx,) = intg.step(intg.tcurr, intg.dt)[:1]
        intg.idxcurr = idx
        intg.tcurr += intg.dt
        lib.memcpy_dtoh(hbuf.value, bank[idx].data, nbytes, stream)
    lib.event_record(e1, stream)
    lib.event_sync(e1)
    wall_e2e = time.perf_counter() - t0
    barrier()
    te2e_ms = allmax(elapsed(e0, e1))
    lib.host_free(hbuf.value)

    res = dict(
        t_ms=t_ms, te2e_ms=te2e_ms, wall_e2e=wall_e2e, gndofs=gndofs,
        nstages=nstages, finite=finite, clocks=clk.summary(),
        launches=launches_per_step*args.steps, kernels=kernels,
        roofline={'bound': 'hbm', 'kernel': dom,
                  'achieved': round(achieved, 1), 'peak': peak,
                  'unit': 'GB/s', 'frac': round(achieved/peak, 4),
                  'traffic': None, 'peak_source': peak_kind,
                  'alg_bytes_per_launch': int(d['bytes']/d['n']),
                  'avg_launch_us': round(1e3*d['ms']/d['n'], 2)},
        e2e_bytes=nbytes, neles=mesh.spts['hex'].shape[1])
    return res


# ---------------------------------------------------------------------------
# CPU arm (the oracle restatement, bounded sample)
# ---------------------------------------------------------------------------

def run_cpu_sample(n_sample, nrhs):
    """Time the CPU oracle's RHS on an n_sample^3 TGV mesh."""
    import numpy as np

    from pyfr_gb300.cases import ns_tgv
    from pyfr_gb300.solvers.elements import NavierStokesElements
    from tests.oracle_util import disc_for_mesh

    cfg, mesh = ns_tgv(n=n_sample, order=3)
    e = NavierStokesElements('hex', mesh.spts['hex'], cfg)
    u = e.set_ics_from_cfg()
    d = disc_for_mesh(mesh, 3, ns=True)
    c = cfg.items_as('constants', float) | cfg.items_as('solver-interfaces',
                                                       float)
    d.rhs_ns(u, c)
    t0 = time.perf_counter()
    for _ in range(nrhs):
        d.rhs_ns(u, c)
    dt = time.perf_counter() - t0
    ndofs = u.size
    return ndofs*nrhs/dt/1e9, dt, ndofs


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=20)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='b200', choices=['b200', 'reference'])
    ap.add_argument('--n', type=int, default=48)
    ap.add_argument('--dt', type=float, default=5e-4)
    ap.add_argument('--cpu-sample', type=int, default=12)
    args = ap.parse_args()

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
        nrhs = max(1, args.steps // 10)
        vals = []
        for _ in range(args.warmup and 1):
            run_cpu_sample(args.cpu_sample, 1)
        for _ in range(max(1, min(args.steps, 3))):
            v, dt, ndofs = run_cpu_sample(args.cpu_sample, nrhs)
            vals.append(v)
        v = statistics.median(vals)
        sample = (f'{args.cpu_sample}^3-element TGV sample, {nrhs} RHS per '
                  'timing, numpy oracle')
        print(json.dumps({
            'impl': 'reference', 'metric': METRIC, 'value': v,
            'unit': 'GDoF/s', 'n_gpus': args.gpus, 'steps': args.steps,
            'warmup': args.warmup, 'higher_is_better': True,
            'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64',
            'data': 'synthetic', 'config': workload,
            'cpu_baseline': {'value': v, 'unit': 'GDoF/s', 'cores': 1,
                             'kind': 'port', 'sample': sample},
            'e2e': {'value': v, 'unit': 'GDoF/s', 'h2d_bytes_per_step': 0,
                    'd2h_bytes_per_step': 0}}))
        return

    res = run_gpu(args, rank, world)
    if rank != 0:
        return

    nrhs = res['nstages']*args.steps
    value = world*res['gndofs']*nrhs/(res['t_ms']*1e-3)/1e9
    e2e = world*res['gndofs']*nrhs/(res['te2e_ms']*1e-3)/1e9

    cpu_v, cpu_dt, cpu_ndofs = run_cpu_sample(args.cpu_sample, 1)

    out = {
        'metric': METRIC, 'value': value, 'unit': 'GDoF/s',
        'n_gpus': world, 'steps': args.steps, 'warmup': args.warmup,
        'ms_per_step': res['t_ms']/args.steps, 'higher_is_better': True,
        'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64',
        'data': 'synthetic', 'config': workload | {
            'ndofs': res['gndofs'], 'dt': args.dt,
            'parallelism': 'replicas' if world > 1 else 'single-gpu'},
        'finite': res['finite'],
        'clocks': res['clocks'],
        'e2e': {'value': e2e, 'unit': 'GDoF/s',
                'h2d_bytes_per_step': res['e2e_bytes'],
                'd2h_bytes_per_step': res['e2e_bytes']},
        'gpu_launches': res['launches'],
        'roofline': res['roofline'],
        'kernels': res['kernels'],
        'cpu_baseline': {'value': cpu_v, 'unit': 'GDoF/s', 'cores': 1,
                         'kind': 'port',
                         'sample': f'one RHS of the numpy oracle on a '
                                   f'{args.cpu_sample}^3 TGV mesh '
                                   f'({cpu_ndofs} DoF, {cpu_dt:.1f} s)'},
    }
    print(json.dumps(out))


if __name__ == '__main__':
    main()
