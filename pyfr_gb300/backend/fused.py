"""Kernel fusion driven by the graphs' group hints.

``Graph.group(kerns, subs)`` is how the reference's systems declare which
element kernels form a chain that may run back to back on one block of
elements (``pyfr/solvers/baseadvec/system.py:126-132``,
``pyfr/solvers/baseadvecdiff/system.py:174-203``).  The fuser receives the
topologically sorted kernel list and the groups of a graph at commit time
and may replace a recognised chain with one fused kernel.
"""


class Fuser:
    def __init__(self, backend):
        self.backend = backend
        self.patterns = []

    def fuse(self, klist, groups):
        for pat in self.patterns:
            klist = pat(self.backend, klist, groups)
        return klist
