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
* ``baseadvec.kernels.negdivconf`` and ``evalsrcmacros`` with the source
  plugin's macro (``plugins/kernels/source.mako``), its expressions made by
  the reference's own substitution (``oracle.refkernels.source_exprs``);
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

from oracle.refkernels import (GAMMA, RK45_A, RK45_B,  # noqa: E402
                               RK45_BHAT, standard_variants as variants)

NPTS = 96
SENTINEL = -777.0


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
    # Source terms: any solution values (both branches of min and max),
    # coordinates in every quadrant (atan2)
    fam['src'] = dict(tdivtconf=rng.normal(size=(n, 5)),
                      ploc=rng.uniform(-2.0, 2.0, (n, 3)),
                      u=rng.normal(0.5, 1.0, (n, 5)),
                      rcpdjac=rng.uniform(0.5, 2.0, n), t=np.array(0.37))
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
