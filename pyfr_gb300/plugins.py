"""Field integrals (kinetic energy and enstrophy) of the integrate plugin.

``FieldIntegrals(intg)()`` returns the domain integrals of the documented
Taylor-Green integrands of ``[soln-plugin-integrate]``
(``doc/src/plugins/soln-plugin-integrate.rst``): ``E`` = rho*|u|^2 and
``enst`` = rho*|curl u|^2, plus the volume ``vol``, using the solution-point
quadrature rule with weights times |J| (``pyfr/plugins/fieldeval.py:80-115``).
The gradients come from the system's gradient pass
(``pyfr/solvers/baseadvecdiff/system.py:233-286``).  Everything is
accumulated in FP64; with the mixed-precision integrator the solution is
the FP64 accumulator and the gradients are FP32.
"""

import ctypes as C

import numpy as np

from pyfr_gb300.shapes import tensor_rule


class FieldIntegrals:
    NBLK = 2048

    def __init__(self, intg):
        self.intg = intg
        be = self.backend = intg.backend
        sysm = intg.system
        if not hasattr(sysm, 'compute_grads'):
            raise ValueError('Field integrals need a system with gradients')

        self._edata = []
        for eles in sysm.ele_map.values():
            b = eles.basis
            _, qw = tensor_rule(b.upts_rule, b.order + 1, b.ndims)
            wts = qw[:, None] / eles.rcpdjac_at_np('upts')
            wmat = be.const_matrix(wts, dtype=np.float64, tags={'align'})
            self._edata.append((eles, wmat))

        self._scratch = be.matrix((1, 3*self.NBLK), dtype=np.float64)
        self._out = be.matrix((1, 3), dtype=np.float64)
        be.commit()
        self._host = np.zeros(3)

    def __call__(self):
        intg, be = self.intg, self.backend
        lib, stream = be.lib, be.stream
        sysm = intg.system
        mixed = hasattr(intg, 'acc')

        uidx = 0 if mixed else intg.idxcurr
        sysm.compute_grads(intg.tcurr, uidx)

        total = np.zeros(3)
        for j, (eles, wmat) in enumerate(self._edata):
            u = intg.acc[j] if mixed else sysm.ele_banks[j][uidx]
            g = eles._grad_upts
            args = (eles.ndims, eles.nupts, eles.neles, u.data, u.leaddim,
                    g.data, g.leaddim, wmat.data, wmat.leaddim)
            if g.dtype == np.float32:
                # The mixed integrator may store u - u_ref
                uref = getattr(intg, 'uref', None) if mixed else None
                pu = None if uref is None else uref.ctypes.data
                lib.integrals_f64f32(*args, pu, self._scratch.data, self.NBLK,
                                     self._out.data, stream)
            else:
                lib.integrals_f64(*args, self._scratch.data, self.NBLK,
                                  self._out.data, stream)
            lib.memcpy_dtoh(self._host.ctypes.data, self._out.data, 24, stream)
            be.wait()
            total += self._host

        return {'E': total[0], 'enst': total[1], 'vol': total[2]}
