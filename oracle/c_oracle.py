"""ctypes front end of the C/OpenMP oracle (test infrastructure and CPU
baseline only).  ``COracle(disc, consts, ...)`` takes a numpy
``fr_oracle.Discretisation`` (which supplies operators, metric terms and the
interface pairing) and evaluates the same right-hand side in C with
OpenMP."""

import ctypes as C

import numpy as np

from oracle.build import build, libpath

i32, i64, f64, vp = C.c_int, C.c_int64, C.c_double, C.c_void_p


class CSR(C.Structure):
    _fields_ = [('m', i32), ('k', i32), ('rowptr', vp), ('colidx', vp),
                ('val', vp)]


class Disc(C.Structure):
    _fields_ = [('ndims', i32), ('nvars', i32), ('nupts', i32),
                ('nfpts', i32), ('neles', i32),
                ('M0', CSR), ('M132', CSR), ('M3', CSR), ('M460', CSR),
                ('M6', CSR), ('smats', vp), ('rcpdjac', vp), ('npairs', i64),
                ('lpt', vp), ('le', vp), ('rpt', vp), ('re', vp), ('nl', vp),
                ('gamma', f64), ('mu', f64), ('pr', f64), ('beta', f64),
                ('tau', f64), ('rsolver', i32)]


def _csr(a, keep):
    a = np.asarray(a, dtype=float)
    rows, cols = np.nonzero(a)
    rowptr = np.zeros(a.shape[0] + 1, dtype=np.int32)
    np.add.at(rowptr, rows + 1, 1)
    rowptr = np.cumsum(rowptr).astype(np.int32)
    colidx = cols.astype(np.int32)
    val = a[rows, cols].copy()
    keep += [rowptr, colidx, val]
    return CSR(a.shape[0], a.shape[1], rowptr.ctypes.data, colidx.ctypes.data,
               val.ctypes.data)


class COracle:
    def __init__(self, disc, consts, rsolver='rusanov', variant='strict'):
        build()
        self._lib = lib = C.CDLL(str(libpath(variant)))
        lib.fro_rhs.argtypes = [C.POINTER(Disc), i32, vp, vp, vp]
        lib.fro_scratch_size.argtypes = [C.POINTER(Disc)]
        lib.fro_scratch_size.restype = i64
        lib.fro_integrals.argtypes = [C.POINTER(Disc), vp, vp, vp, vp]

        d = disc
        self.ndims, self.nupts, self.neles = d.ndims, d.nupts, d.neles
        self.nvars = d.ndims + 2
        keep = self._keep = []
        ns = 'M460' in d.ops

        smats = np.ascontiguousarray(d.smats_u.transpose(3, 0, 1, 2))  # e,p,i,j
        rcp = np.ascontiguousarray((1.0/d.djac_u).T)
        pl, pr = d.pl.astype(np.int64), d.pr.astype(np.int64)
        lpt, le = np.ascontiguousarray(pl[:, 0]), np.ascontiguousarray(pl[:, 1])
        rpt, re = np.ascontiguousarray(pr[:, 0]), np.ascontiguousarray(pr[:, 1])
        nl = np.ascontiguousarray(d.nl.T)
        keep += [smats, rcp, lpt, le, rpt, re, nl]

        zero = np.zeros((1, 1))
        ops = {k: d.ops.get(k, zero) for k in ('M0', 'M132', 'M3', 'M460', 'M6')}
        self.disc = Disc(
            d.ndims, self.nvars, d.nupts, d.nfpts, d.neles,
            _csr(ops['M0'], keep), _csr(ops['M132'], keep),
            _csr(ops['M3'], keep), _csr(ops['M460'], keep),
            _csr(ops['M6'], keep), smats.ctypes.data, rcp.ctypes.data,
            len(lpt), lpt.ctypes.data, le.ctypes.data, rpt.ctypes.data,
            re.ctypes.data, nl.ctypes.data, consts['gamma'],
            consts.get('mu', 0.0), consts.get('Pr', 1.0),
            consts.get('ldg-beta', 0.5), consts.get('ldg-tau', 0.0),
            {'rusanov': 0, 'hllc': 1}[rsolver])
        self.ns = ns
        self._scratch = np.empty(lib.fro_scratch_size(C.byref(self.disc)))

    def rhs_native(self, ue):
        """RHS on element-major data u[e][pt][var] (no layout change)."""
        r = np.empty_like(ue)
        self._lib.fro_rhs(C.byref(self.disc), int(self.ns), ue.ctypes.data,
                          r.ctypes.data, self._scratch.ctypes.data)
        return r

    def integrals_native(self, ue, qw):
        """(kinetic energy, enstrophy, volume) integrals of a 3-D
        Navier-Stokes solution u[e][pt][var] with solution-point weights qw
        (times |J|)."""
        out = np.zeros(3)
        qw = np.ascontiguousarray(qw, dtype=float)
        if self._lib.fro_integrals(C.byref(self.disc), ue.ctypes.data,
                                   qw.ctypes.data, self._scratch.ctypes.data,
                                   out.ctypes.data):
            raise ValueError('Integrals need a 3-D Navier-Stokes system')
        return out

    def rhs(self, u):
        """RHS on (nupts, nvars, neles) data, as the numpy oracle."""
        ue = np.ascontiguousarray(u.transpose(2, 0, 1))
        return self.rhs_native(ue).transpose(1, 2, 0)
