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


class WriterPlugin:
    """Solution output of ``[soln-plugin-writer]`` (``pyfr/plugins/
    writer.py:8-160``): every ``dt-out`` of simulated time (and at the
    start of a run that is not a restart) the solution is written to
    ``basedir/basename`` (formatted with the time ``t`` and the output
    count ``n``; the ``.pyfrs`` extension is added), with the
    configuration chain, the run statistics and the integrator's
    serialised state, and with ``write-gradients`` the physical gradients.
    ``files`` lists what was written."""

    name = 'writer'

    def __init__(self, intg, cfgsect='soln-plugin-writer'):
        from pathlib import Path

        from pyfr_gb300.native import file_path_gen

        cfg = intg.cfg
        self._grads = cfg.getbool(cfgsect, 'write-gradients', False)
        if self._grads and not hasattr(intg.system, 'compute_grads'):
            raise ValueError('Gradient output needs a system with '
                             'gradients')
        basedir = Path(cfg.get(cfgsect, 'basedir', '.')).absolute()
        basename = cfg.get(cfgsect, 'basename')
        if not basename.endswith('.pyfrs'):
            basename += '.pyfrs'
        self._fgen = file_path_gen(basedir, basename)
        next(self._fgen)

        emap = intg.system.ele_map
        self.fields = list(next(iter(emap.values())).convars)
        self._upts = {et: e.basis.upts for et, e in emap.items()}

        self.dt_out = cfg.getfloat(cfgsect, 'dt-out')
        self.tol = 5*intg.dtmin
        self.tout_last = intg.tcurr
        intg.call_plugin_dt(intg.tcurr, self.dt_out)
        if not intg.isrestart:
            self.tout_last -= self.dt_out
        self.files = []

    def __call__(self, intg):
        if intg.tcurr - self.tout_last < self.dt_out - self.tol:
            return
        self.write(intg)
        self.tout_last = intg.tcurr

    def write(self, intg):
        from pyfr_gb300.inifile import Inifile
        from pyfr_gb300.native import write_soln

        stats = Inifile()
        stats.set('data', 'prefix', 'soln')
        intg.collect_stats(stats)
        path = self._fgen.send(intg.tcurr)
        sysm = intg.system
        grads = None
        if self._grads:
            # (the mixed-precision integrator's FP32 input is refreshed
            # from its FP64 solution at every step start)
            uidx = 0 if hasattr(intg, 'acc') else intg.idxcurr
            sysm.compute_grads(intg.tcurr, uidx)
            gl = sysm.grad_upts()
            if getattr(intg, 'uref', None) is not None:
                # Gradients of the shifted variables q: grad E = grad q_E +
                # h_ref grad rho
                for g in gl:
                    g[:, :, -1] += intg.hs_ref*g[:, :, 0]
            grads = dict(zip(sysm.ele_types, gl))
        write_soln(path, sysm.mesh, dict(zip(sysm.ele_types, intg.soln)),
                   self._upts, self.fields, intg.cfg, stats,
                   prevcfgs=intg.prevcfgs, state=intg.serialise(),
                   grads=grads)
        self.files.append(path)
