"""Bit-level checks of the mixed-precision stage kernel and the FP64->FP32
narrowing, which convert on the integer pipes: results must equal IEEE 754
round-to-nearest-even conversions (numpy's astype) bit for bit, including
ties, zeros, subnormal, infinite and NaN values, ragged lengths and
unaligned pointers; and the shifted error norm and field integrals must
equal the unshifted ones."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def be():
    import __graft_entry__ as ge
    from pyfr_gb300.backend import B200Backend
    from pyfr_gb300.inifile import Inifile
    ge.build_library()
    return B200Backend(Inifile())


class Dev:
    """Raw device buffer with host round trips."""
    def __init__(self, be, ary, pad=64):
        self.lib, self.stream = be.lib, be.stream
        self.ary = np.ascontiguousarray(ary)
        p = C.c_void_p()
        self.lib.malloc(C.byref(p), self.ary.nbytes + pad)
        self.base = p.value
        self.ptr = self.base

    def at(self, off_elems):
        self.ptr = self.base + off_elems*self.ary.itemsize
        return self

    def put(self):
        self.lib.memcpy_htod(self.ptr, self.ary.ctypes.data, self.ary.nbytes,
                             self.stream)
        return self

    def take(self):
        out = np.empty_like(self.ary)
        self.lib.memcpy_dtoh(out.ctypes.data, self.ptr, out.nbytes,
                             self.stream)
        self.lib.stream_sync(self.stream)
        return out

    def free(self):
        self.lib.free(self.base)


def _f64_edge_values(rng, n):
    """FP64 values spread over and beyond the FP32 range, with exact
    FP32 rounding ties and values next to them."""
    mags = 10.0**rng.uniform(-50, 50, size=n)
    x = rng.choice([-1.0, 1.0], size=n)*mags
    f = rng.normal(size=n).astype(np.float32)
    half = np.spacing(np.abs(f)).astype(np.float64)/2
    ties = f.astype(np.float64) + half
    near = np.nextafter(ties, np.inf)
    big = np.array([3.4028234663852886e38, 3.4028235677973366e38,
                    3.4028235677973362e38, 1.1754943508222875e-38,
                    1.1754942e-38, 1.4e-45, 7e-46, 0.0, -0.0, np.inf,
                    -np.inf, np.nan, 1e300, -1e-300])
    return np.concatenate([x, ties, -ties, near, big])


def _same_bits(a, b):
    nan = np.isnan(a) & np.isnan(b)
    return np.all((a.view(np.uint32 if a.dtype == np.float32 else np.uint64)
                   == b.view(np.uint32 if b.dtype == np.float32
                             else np.uint64)) | nan)


@pytest.mark.parametrize('offset', [0, 1])
def test_narrowing_is_round_to_nearest_even(be, offset):
    rng = np.random.default_rng(11)
    src = _f64_edge_values(rng, 20000)
    with np.errstate(over='ignore'):
        ref = src.astype(np.float32)
    d = Dev(be, src).at(offset).put()
    o = Dev(be, np.zeros(len(src), np.float32)).at(offset)
    be.lib.cast_f64_f32(len(src), d.ptr, o.ptr, 0, None, be.stream)
    got = o.take()
    d.free(), o.free()
    assert _same_bits(got, ref)


def _rhs_values(rng, n):
    r = rng.normal(size=n).astype(np.float32)
    r[::17] = 0.0
    r[1::17] = -0.0
    r[2::31] = np.float32(1e-40)                   # subnormal
    r[3::31] = np.float32(-3e-39)
    return r


@pytest.mark.parametrize('n,offset', [(4096, 0), (1001, 0), (1003, 1)])
@pytest.mark.parametrize('errest', [0, 1])
def test_rkmixed_stage_bit_exact(be, n, offset, errest):
    """dt = 1 with b = 1 and a = 1/2 makes every FMA of the stage a single
    correctly rounded sum, which numpy reproduces exactly:
    acc' = acc + f64(R), input = f32(acc) + R/2, last input = f32(acc')."""
    rng = np.random.default_rng(n + offset)
    acc0 = rng.normal(size=n)*10.0**rng.integers(-3, 3, size=n)
    acc0[::13] = 0.0
    r = _rhs_values(rng, n)
    rerr0 = rng.normal(size=n)

    for stage, nstages in [(0, 5), (2, 5), (4, 5)]:
        last = stage == nstages - 1
        A = Dev(be, acc0).at(offset).put()
        R = Dev(be, r).at(offset).put()
        U = Dev(be, np.zeros(n, np.float32)).at(offset).put()
        RO = Dev(be, np.zeros(n)).at(offset).put()
        RE = Dev(be, rerr0).at(offset).put()
        be.lib.rkmixed_f64f32(n, stage, nstages, errest, 1.0, 0.5, 1.0, 0.25,
                              A.ptr, R.ptr, U.ptr,
                              RO.ptr if errest else None,
                              RE.ptr if errest else None, be.stream)
        acc, u, rold, rerr = A.take(), U.take(), RO.take(), RE.take()
        for m in (A, R, U, RO, RE):
            m.free()

        r64 = r.astype(np.float64)
        nacc = acc0 + r64
        assert _same_bits(acc, nacc)
        if last:
            assert _same_bits(u, nacc.astype(np.float32))
        else:
            assert _same_bits(u, acc0.astype(np.float32) +
                              np.float32(0.5)*r)
        if errest:
            if stage == 0:
                assert _same_bits(rold, acc0)
                assert _same_bits(rerr, 0.25*r64)
            else:
                assert _same_bits(rerr, rerr0 + 0.25*r64)


def test_shifted_error_norm(be):
    """The error norm of a solution stored as q = T(u - u_ref) (energy
    component dE - h*drho), with its error estimate in q, equals the norm
    of u and of its error."""
    rng = np.random.default_rng(5)
    shape = (16, 5, 45)
    uref = np.array([1.0, 0.0, 0.0, 0.0, 178.5])
    h = 250.0
    cur = rng.normal(size=shape) + uref[None, :, None]
    err = 1e-6*rng.normal(size=shape)
    q = cur - uref[None, :, None]
    q[:, -1] -= h*q[:, 0]
    eq = err.copy()
    eq[:, -1] -= h*eq[:, 0]
    C_ = be.matrix(shape, cur, tags={'align'})
    S = be.matrix(shape, q, tags={'align'})
    E = be.matrix(shape, err, tags={'align'})
    EQ = be.matrix(shape, eq, tags={'align'})
    be.commit()
    atols = [1e-6, 2e-6, 3e-6, 4e-6, 5e-6]
    ks = [be.kernel('errest', C_, E, atols),
          be.kernel('errest', S, EQ, atols, uref=uref, hcoef=h)]
    vals = []
    for k in ks:
        k.bind(rtol=1e-5)
        k.run(be.stream)
        be.wait()
        vals.append(k.retval[0])
    ref = np.sum((err/(np.array(atols)[None, :, None] +
                       1e-5*np.abs(cur)))**2)
    assert abs(vals[0] - ref) <= 1e-12*ref
    assert abs(vals[1] - ref) <= 1e-12*ref
