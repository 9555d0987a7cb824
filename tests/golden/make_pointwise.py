"""Golden vectors for the pointwise kernels, computed by the reference's own
kernel sources.

The reference's ``.mako`` kernels are rendered to C and compiled by
``oracle/refkernels.py`` (into ``oracle/_ref/``), then evaluated here on
seeded random but physically valid inputs; inputs and outputs are written
to ``pointwise.npz`` next to this script.  Run where the reference checkout
is present (``PYFR_REFERENCE``, default ``/root/reference``, or the first
argument):

  python tests/golden/make_pointwise.py [reference-root]

Kernels covered (reference module, variants):

* ``euler.kernels.tflux`` (2-D, 3-D), ``euler.kernels.wavespeed``;
* ``euler.kernels.intcflux`` with every Riemann solver of
  ``euler/kernels/rsolvers`` (rusanov, hllc, hll, roe, roem, exact);
* ``navstokes.kernels.tflux`` fused (constant viscosity and Sutherland);
* ``navstokes.kernels.intcflux`` for beta in {1/2, 0, -1/2}, tau in
  {0.1, 0}, Rusanov and HLLC (plus the other solvers at beta = 1/2);
* ``navstokes.kernels.intconu`` for the three betas;
* ``baseadvecdiff.kernels.gradcoru``, ``baseadvec.kernels.negdivconf``;
* ``integrators.explicit.kernels.rkvdh2`` for every RK45 stage, with and
  without the embedded error register.
"""

import json
import os
from pathlib import Path
import sys

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path.insert(0, str(REPO))

GAMMA = 1.4
NPTS = 96
RSOLVERS = ['rusanov', 'hllc', 'hll', 'roe', 'roem', 'exact']
SENTINEL = -777.0

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


def states(rng, n, nd):
    """Conserved states with density in [0.5, 2], pressure in [0.4, 2.5]
    and velocities up to supersonic."""
    rho = rng.uniform(0.5, 2.0, n)
    v = rng.normal(0.0, 0.7, (n, nd))
    p = rng.uniform(0.4, 2.5, n)
    E = p/(GAMMA - 1) + 0.5*rho*(v**2).sum(1)
    return np.column_stack([rho, rho[:, None]*v, E])


def normals(rng, n, nd):
    """Scaled normals: random directions plus axis-aligned and near-axis
    ones (every branch of the 3-D normal-frame transform)."""
    d = rng.normal(size=(n, nd))
    if nd == 3:
        special = np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, 0, -1],
                            [0.995, 0.07, 0.07], [0.995, -0.02, 0.09],
                            [-0.995, 0.09, 0.02], [0.999, 0.04, -0.01]])
    else:
        special = np.array([[1, 0], [0, -1], [-1, 0], [0.6, 0.8]])
    d[:len(special)] = special
    d /= np.linalg.norm(d, axis=1)[:, None]
    return d*rng.uniform(0.5, 2.0, n)[:, None]


def smats(rng, n, nd):
    return np.eye(nd)[None] + 0.3*rng.normal(size=(n, nd, nd))


def constants(visc=False, sutherland=False, beta=0.5, tau=0.1):
    c = {'gamma': GAMMA}
    if visc:
        c |= {'mu': 0.05, 'Pr': 0.72, 'ldg-beta': beta, 'ldg-tau': tau}
        if sutherland:
            c |= {'cpTref': 3.0, 'cpTs': 1.2}
    return c


def variants():
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
    e = [b - bh for b, bh in zip(RK45_B, RK45_BHAT)]
    for errest in (False, True):
        for s in range(5):
            v[f'rkvdh2_s{s}_e{int(errest)}'] = (
                'pyfr.integrators.explicit.kernels.rkvdh2', 'rkvdh2',
                dict(nvars=5, stage=s, nstages=5, errest=errest, a=RK45_A,
                     b=RK45_B, e=e), 'rk')
    return v


def inputs(rng):
    fam = {}
    n = NPTS
    for nd in (2, 3):
        nv = nd + 2
        fam[f'euler{nd}_elem'] = dict(u=states(rng, n, nd),
                                      smats=smats(rng, n, nd),
                                      rcpdjac=rng.uniform(0.5, 2.0, n))
        ul, ur = states(rng, n, nd), states(rng, n, nd)
        ur[-8:] = ul[-8:]                     # consistency: F(u, u, n)
        fam[f'euler{nd}_iface'] = dict(ul=ul, ur=ur, nl=normals(rng, n, nd))
        fam[f'ns{nd}_elem'] = dict(u=states(rng, n, nd),
                                   gradu=rng.normal(0, 0.5, (n, nd, nv)),
                                   smats=smats(rng, n, nd),
                                   rcpdjac=rng.uniform(0.5, 2.0, n))
        ul, ur = states(rng, n, nd), states(rng, n, nd)
        ur[-8:] = ul[-8:]
        fam[f'ns{nd}_iface'] = dict(ul=ul, ur=ur, nl=normals(rng, n, nd),
                                    gradul=rng.normal(0, 0.5, (n, nd, nv)),
                                    gradur=rng.normal(0, 0.5, (n, nd, nv)))
    fam['conu'] = dict(ulin=states(rng, n, 3), urin=states(rng, n, 3),
                       ulout=np.full((n, 5), SENTINEL),
                       urout=np.full((n, 5), SENTINEL))
    fam['negdivconf'] = dict(tdivtconf=rng.normal(size=(n, 5)),
                             rcpdjac=rng.uniform(0.5, 2.0, n))
    fam['rk'] = dict(r1=rng.normal(size=(n, 5)), r2=rng.normal(size=(n, 5)),
                     rold=np.full((n, 5), SENTINEL),
                     rerr=rng.normal(size=(n, 5)), dt=np.array(2.5e-3))
    return fam


def main(root=None):
    if root:
        os.environ['PYFR_REFERENCE'] = root
    from oracle.refkernels import RefLibrary

    var = variants()
    lib = RefLibrary({k: (m, kn, tp, None) for k, (m, kn, tp, _) in
                      var.items()})
    rng = np.random.default_rng(20261204)
    fam = inputs(rng)

    out = {}
    for f, arrs in fam.items():
        for a, x in arrs.items():
            out[f'in:{f}:{a}'] = x
    meta = {}
    for cname, (mod, kname, tplargs, f) in var.items():
        k = lib.kernels[cname]
        args = {a.name: fam[f][a.name] for a in k.vectargs
                if a.name in fam[f]}
        scal = {a.name: fam[f][a.name] for a in k.scalargs}
        res = lib(cname, NPTS, **args, **scal)
        for a in k.vectargs:
            if a.intent != 'in':
                out[f'out:{cname}:{a.name}'] = res[a.name]
        tp = {k2: v2 for k2, v2 in tplargs.items()}
        meta[cname] = dict(module=mod, kernel=kname, family=f,
                           tplargs=tp,
                           outputs=[a.name for a in k.vectargs
                                    if a.intent != 'in'])

    out['meta'] = np.array(json.dumps(meta, default=float))
    np.savez_compressed(HERE / 'pointwise.npz', **out)
    print(f'{len(var)} kernels, {sum(x.size for x in out.values())} values '
          f'-> {HERE / "pointwise.npz"} (library {lib.path})')


if __name__ == '__main__':
    main(sys.argv[1] if len(sys.argv) > 1 else None)
