"""Kernel fusion driven by the graphs' group hints.

``Graph.group(kerns, subs)`` is how the reference's systems declare which
element kernels form a chain that may run back to back on one block of
elements (``pyfr/solvers/baseadvec/system.py:126-132``,
``pyfr/solvers/baseadvecdiff/system.py:174-203``).  The fuser receives the
topologically sorted kernel list and the groups of a graph at commit time
and replaces each recognised chain with one fused kernel.

Pattern (with fused operator applies, ``fuse-operators``):

* the divergence chain of one element type, ``tdivtpcorf`` (R = (M1 -
  M3 M2) F), ``tdivtconf`` (R += M3 Fc) and ``negdivconf`` (R = -R/|J|, no
  source terms), becomes one tensor-core apply of the two operators side
  by side, R = -(1/|J|)((M1 - M3 M2) F + M3 Fc): the partial divergence
  never goes to memory and two passes over R go away.  PyFR's own Euler
  system groups exactly these kernels
  (``pyfr/solvers/baseadvec/system.py:126-132``); this package's own systems
  build the fused apply directly.
"""

from pyfr_gb300.backend.types import Kernel


def _mul_meta(k):
    m = k.meta
    if k.name != 'mul' or m.get('a') is None or m.get('a2') is not None:
        return None
    if m.get('nbatch', 1) != 1 or m.get('rowscale') is not None:
        return None
    return m


def divergence_chain(backend, klist, groups):
    """tdivtpcorf + tdivtconf + negdivconf -> one ``mul_cat`` apply."""
    from pyfr_gb300.backend.base import NotSuitableError

    if not backend.fuse_operators:
        return klist
    out = list(klist)
    for kerns, _ in groups:
        ks = [k for k in kerns if isinstance(k, Kernel)]
        negs = [k for k in ks if k.name == 'negdivconf']
        muls = [k for k in ks if _mul_meta(k) is not None]
        if len(negs) != 1 or len(muls) != 2:
            continue
        neg = negs[0]
        r, rj = neg.meta.get('tdivtconf'), neg.meta.get('rcpdjac')
        if r is None or rj is None or neg.meta['tplargs'].get('src_macros'):
            continue
        k1, k2 = sorted(muls, key=lambda k: k.meta['beta'])
        m1, m2 = k1.meta, k2.meta
        if not (m1['out'] is r and m2['out'] is r and m1['beta'] == 0.0 and
                m2['beta'] == 1.0 and m1['alpha'] == 1.0 and
                m2['alpha'] == 1.0):
            continue
        if any(k not in out for k in (k1, k2, neg)):
            continue
        i1, i2, i3 = (out.index(k) for k in (k1, k2, neg))
        if not i1 < i2 < i3:
            continue
        try:
            fused = backend.kernel('mul_cat', m1['a'], m1['b'], m2['a'],
                                   m2['b'], out=r, alpha=-1.0, rowscale=rj)
        except NotSuitableError:
            continue
        # In the place of negdivconf: after everything tdivtconf waited
        # for (the common flux), before every reader of the result
        out[i3] = fused
        out.remove(k1)
        out.remove(k2)
    return out


class Fuser:
    def __init__(self, backend):
        self.backend = backend
        self.patterns = [divergence_chain]

    def fuse(self, klist, groups):
        for pat in self.patterns:
            klist = pat(self.backend, klist, groups)
        return klist
